"""Benchmark of the ERI + Fock (J/K) build on one GB300.

Workload: benzene C6H6 RHF/6-31G (D6h, C-C 1.39 A, C-H 1.09 A), 66 basis
functions, 2,445,366 unique contracted function quartets.  One step = one
integral-direct Fock build G = J - K/2 from a density resident in HBM (the
converged SCF density of the molecule).

Metric: ERI+Fock quartets/s = unique function quartets / build time (screened
quartets count in the numerator for every path), plus the SCF wall time.
``value`` is the plain FP64 path (the drop-in); the mixed FP32/FP64 path and
its energy error against the FP64 result are reported beside it.

Timing: W warm-up builds, then K builds, each bracketed by CUDA events on the
stream the library launches on; between builds a 256 MB buffer is written to
flush the 129 MB L2 (outside the events).  ``e2e`` times the C-ABI call with
host buffers (fock_build_jk: H2D of D, build, D2H of G).

``--impl reference`` times the reference's algorithm (the CPU restatement in
oracle/: recursive E/R, per-function primitive loops, dense N^4 tensor with
1e-6 zeroing, serial electron_terms + G loops) on all host cores, on a
bounded sample of the outer w loop.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# 32 hardware work queues for this process's CUDA context (the library's own
# default, which only takes effect before the context exists; torch creates it
# first here): the build graph's class launches are up to 32 parallel branches
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fock-rs_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "ERI+Fock quartets/s (C6H6 RHF/6-31G Fock build)"
UNIT = "quartets/s"
# SCF start of every bench workload: superposition of atomic densities (the
# core guess leaves (H2O)32 and 2 of the 512 clusters unconverged), no level shift
SCF_GUESS_NAME = "sad"
BATCH_LEVEL_SHIFT = 0.0  # Eh
MIXED_CURVE = (1.0, 0.1, 0.01, 1e-3, 1e-4)  # mixed thresholds of the batch's speed / accuracy curve
BUILD_DRAM_BYTES_NCU = 5.1e6  # DRAM bytes per benzene FP64 build under ncu (launch list: 4 builds / 4)
WORKLOAD = {"workload": "C6H6 RHF/6-31G integral-direct Fock build (G = J - K/2)", "molecule": "benzene D6h",
            "basis": "6-31G", "n_basis": 66, "unique_quartets": 2445366, "l2": "flushed between steps (256 MB write)"}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def benzene_atoms():
    from fock_gb300 import basis as B
    from fock_gb300 import molecules as M
    Zs, xyz = M.benzene()
    return B.build_atoms("6-31G", Zs, xyz)


def cpu_reference(steps, warmup, threads=0):
    """Reference algorithm on the host cores; one step = the sampled outer-w
    iterations of from_basis + the full electron_terms and G loops.  The w
    loop is the parallel one (rayon in the reference, OpenMP here), so the
    sample keeps at least 4 w iterations per thread: every core stays busy."""
    import oracle
    oracle.build()
    atoms = benzene_atoms()
    ob = oracle.OracleBasis(atoms)
    n = ob.n
    rng = np.random.default_rng(0)
    Cm = rng.normal(size=(n, 21)) / np.sqrt(n)
    D = 2.0 * Cm @ Cm.T
    nthreads = threads or oracle.max_threads()
    stride = max(1, n // (4 * nthreads))
    rates, tf_all = [], []
    total_unique = WORKLOAD["unique_quartets"]
    for it in range(warmup + steps):
        w0 = (it * 7) % stride
        cnt, te, tf = oracle.ref_build_timed(ob, D, oracle.REFCOMPAT, w_begin=w0, w_stride=stride,
                                             full_fock=(it == warmup), threads=nthreads)
        if it >= warmup:
            rates.append(cnt / te)
            if tf > 0:
                tf_all.append(tf)
    rate = statistics.median(rates)
    t_eri = total_unique / rate
    t_fock = tf_all[0] if tf_all else 0.0
    value = total_unique / (t_eri + t_fock)
    return value, {"kind": "port", "cores": nthreads,
                   "sample": "outer-w iterations w0, w0+%d, ... of from_basis (about 1/%d of the quartets) per step, "
                             "literal recursive E/R, 1e-6 zeroing; electron_terms + G loops timed in full once "
                             "(%.2f s); full-build time extrapolated by quartet count" % (stride, stride, t_fock),
                   "eri_quartets_per_s": rate, "est_full_build_s": t_eri + t_fock}


def _event_times(torch, stream, fn, k, w, flush):
    """Device times (ms) of k calls of fn on ``stream`` after w warm-up calls, L2 flushed before each."""
    with torch.cuda.stream(stream):
        for _ in range(w):
            fn()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for e0, e1 in ev:
            flush.fill_(1.0)
            e0.record(stream)
            fn()
            e1.record(stream)
    stream.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


def batch_workload(torch, F, L, local, flush, steps=3, warmup=3, spot=6):
    """512 water clusters (H2O)_n, n ~ U{1..8} (seed 0), RHF/6-31G, one batch context.

    Mixed-precision batched SCF (final iterations FP64) gives the converged
    densities; FP64 and mixed batched Fock builds are timed at those densities;
    the mixed build's energy error per molecule is 1/2 sum D (G_mixed - G_fp64);
    ``spot`` molecules are re-solved alone in FP64 and compared with the batch."""
    from fock_gb300 import basis as B, molecules as M
    batch = M.water_cluster_batch(512, seed=0)
    mols = [B.build_atoms("6-31G", Zs, xyz) for Zs, xyz in batch]
    kw = dict(guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, epsilon=1e-8, max_iters=100,
              level_shift=BATCH_LEVEL_SHIFT, sign_convention=L.FOCK_SIGN_STANDARD, device=local)
    out = {"workload": "512 water clusters (H2O)_n, n~U{1..8} seed 0, RHF/6-31G, one batched context"}
    # warm-up: a 2-iteration batched SCF over one cluster of every size loads the
    # cuBLAS / cuSOLVER kernels of every matrix shape (one-time lazy loading)
    sizes = {}
    for i, (Zs, _) in enumerate(batch):
        sizes.setdefault(len(Zs), i)
    with F.FockBatch([mols[i] for i in sorted(sizes.values())], **dict(kw, max_iters=2)) as wb:
        wb.scf()
    t0 = time.perf_counter()
    b = F.FockBatch(mols, **kw)
    out["create_s"] = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    b.set_precision(L.FOCK_PREC_MIXED, F.options().mixed_threshold)
    t0 = time.perf_counter()
    rc, res, dens = b.scf(densities=True)
    torch.cuda.synchronize()
    out["scf_mixed"] = {"rc": rc, "wall_s": time.perf_counter() - t0, "fock_s": res[0].fock_seconds,
                        "fock_builds": res[0].fock_builds, "converged": sum(r.converged for r in res),
                        "iterations_max": max(r.iterations for r in res),
                        "level_shift_eh": BATCH_LEVEL_SHIFT, "guess": SCF_GUESS_NAME}
    D = torch.zeros(b.total, dtype=torch.float64, device="cuda")
    for off, n, Dm in zip(b.offsets, b.nbf, dens):
        D[off:off + n * n] = torch.from_numpy(Dm.reshape(-1))
    G = torch.zeros_like(D)
    st = b.stats()
    nq = st["function_quartets_unique"]
    out["unique_quartets"] = nq
    res_prec = {}
    Gs = {}
    for name, prec in (("fp64", L.FOCK_PREC_FP64), ("mixed", L.FOCK_PREC_MIXED)):
        b.set_precision(prec, F.options().mixed_threshold)
        l0 = b.launch_count()
        t = _event_times(torch, stream, lambda: b.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
        ms = sum(t) / len(t)
        res_prec[name] = {"ms_per_build": ms, "quartets_per_s": nq / (ms * 1e-3),
                          "launches_per_build": (b.launch_count() - l0) // (steps + warmup)}
        Gs[name] = G.clone()
    res_prec["mixed"]["speedup_vs_fp64"] = res_prec["fp64"]["ms_per_build"] / res_prec["mixed"]["ms_per_build"]
    # autotuned launch parameters of the mixed batched build (fock_batch_autotune, fresh cache)
    import tempfile
    from fock_gb300.tuning import autotune
    b.set_precision(L.FOCK_PREC_MIXED, F.options().mixed_threshold)
    with tempfile.TemporaryDirectory() as td:
        tuned = autotune(b, D.data_ptr(), reps=2, cache_path=os.path.join(td, "tune.json"), batch=True)
    t = _event_times(torch, stream, lambda: b.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
    ms_t = sum(t) / len(t)
    res_prec["mixed_autotuned"] = {"ms_per_build": ms_t, "quartets_per_s": nq / (ms_t * 1e-3),
                                   "speedup_vs_fp64": res_prec["fp64"]["ms_per_build"] / ms_t,
                                   "tuning": {k: tuned[k] for k in ("prims_per_slice", "prims_per_slice_fp32",
                                                                    "block_threads", "persistent")}}
    dG = Gs["mixed"] - Gs["fp64"]
    de = [0.5 * float((D[o:o + n * n] * dG[o:o + n * n]).sum().item()) for o, n in zip(b.offsets, b.nbf)]
    res_prec["mixed"]["max_single_build_energy_error_eh"] = max(abs(x) for x in de)
    # speed / accuracy curve of one mixed build over the threshold (density-weighted split)
    curve = []
    for th in MIXED_CURVE:
        b.set_precision(L.FOCK_PREC_MIXED, th)
        t = _event_times(torch, stream, lambda: b.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
        ms_c = sum(t) / len(t)
        dGc = G - Gs["fp64"]
        dec = [0.5 * float((D[o:o + n * n] * dGc[o:o + n * n]).sum().item()) for o, n in zip(b.offsets, b.nbf)]
        stc = b.stats()
        curve.append({"mixed_threshold": th, "ms_per_build": ms_c,
                      "speedup_vs_fp64": res_prec["fp64"]["ms_per_build"] / ms_c,
                      "max_single_build_energy_error_eh": max(abs(x) for x in dec),
                      "fp32_shell_quartets": stc["shell_quartets_fp32"], "fp64_shell_quartets": stc["shell_quartets_fp64"]})
    res_prec["mixed_threshold_curve"] = curve
    ok = [c for c in curve if c["max_single_build_energy_error_eh"] <= 1e-6]
    res_prec["best_speedup_at_1e-6_eh_per_build"] = max((c["speedup_vs_fp64"] for c in ok), default=None)
    b.set_precision(L.FOCK_PREC_MIXED, F.options().mixed_threshold)
    out.update(res_prec)
    # spot check: molecules solved alone in FP64 against the batched mixed SCF
    idx = np.linspace(0, len(mols) - 1, spot).astype(int)
    worst = 0.0
    for i in idx:
        r = F.try_scf(mols[i], 100, 1e-8, 0, **{k: v for k, v in kw.items() if k not in ("max_iters", "epsilon")})
        if r is not None and r.converged and res[i].converged:
            worst = max(worst, abs(r.total_energy - res[i].total_energy))
    out["scf_mixed"]["max_abs_energy_error_vs_single_fp64_eh"] = worst
    out["scf_mixed"]["spot_checked_molecules"] = [int(i) for i in idx]
    # the same batched SCF in plain FP64, for the SCF-time ratio of the metric
    b.set_precision(L.FOCK_PREC_FP64, F.options().mixed_threshold)
    t0 = time.perf_counter()
    rc64, res64, _ = b.scf(densities=True)
    torch.cuda.synchronize()
    wall64 = time.perf_counter() - t0
    out["scf_fp64"] = {"rc": rc64, "wall_s": wall64, "fock_s": res64[0].fock_seconds,
                       "fock_builds": res64[0].fock_builds, "converged": sum(r.converged for r in res64),
                       "iterations_max": max(r.iterations for r in res64)}
    out["scf_mixed"]["speedup_vs_fp64_scf"] = wall64 / out["scf_mixed"]["wall_s"]
    out["scf_mixed"]["max_abs_energy_error_vs_batched_fp64_eh"] = max(
        abs(a.total_energy - r.total_energy) for a, r in zip(res, res64) if a.converged and r.converged)
    b.close()
    return out


def benzene_builds(torch, F, L, local, flush, steps=3, warmup=3, precision=None):
    """Fock builds of the headline workload alone (no SCF): for launch lists and captures."""
    precision = L.FOCK_PREC_FP64 if precision is None else precision
    ctx = F.FockContext(benzene_atoms(), sign_convention=L.FOCK_SIGN_STANDARD, device=local, precision=precision)
    n = ctx.n
    rng = np.random.default_rng(0)
    Cm = rng.normal(size=(n, 21)) / np.sqrt(n)
    D = torch.tensor(2.0 * Cm @ Cm.T, device="cuda")
    G = torch.empty_like(D)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    t = _event_times(torch, stream, lambda: ctx.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
    st = ctx.stats()
    ctx.close()
    return {"ms_per_build": sum(t) / len(t), "launches_per_build": st["launches_per_build"],
            "flops_fp64": st["flops_fp64"]}


def water32_workload(torch, F, L, local, flush, steps=3, warmup=3, builds_only=False):
    """(H2O)_32 cluster (seed 0), RHF/6-31G* with Cartesian d on O: 608 functions.
    FP64 and mixed Fock builds at a density of 160 random orthonormal-ish orbitals."""
    from fock_gb300 import basis as B, molecules as M
    Zs, xyz = M.water_cluster(32, seed=0)
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    ctx = F.FockContext(atoms, sign_convention=L.FOCK_SIGN_STANDARD, device=local)
    n = ctx.n
    rng = np.random.default_rng(0)
    Cm = rng.normal(size=(n, 160)) / np.sqrt(n)
    D = torch.tensor(2.0 * Cm @ Cm.T, device="cuda")
    G = torch.empty_like(D)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    st = ctx.stats()
    nq = st["function_quartets_unique"]
    out = {"workload": "(H2O)32 seed 0, RHF/6-31G*, %d functions" % n, "unique_quartets": nq}
    Gs = {}
    for name, prec in (("fp64", L.FOCK_PREC_FP64), ("mixed", L.FOCK_PREC_MIXED)):
        ctx.set_precision(prec, F.options().mixed_threshold)
        t = _event_times(torch, stream, lambda: ctx.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
        ms = sum(t) / len(t)
        out[name] = {"ms_per_build": ms, "quartets_per_s": nq / (ms * 1e-3)}
        if prec == L.FOCK_PREC_FP64:  # model FP64 flops of the plan over the build time
            out[name]["tflops_fp64"] = ctx.stats()["flops_fp64"] / (ms * 1e-3) / 1e12
        Gs[name] = G.clone()
    out["mixed"]["speedup_vs_fp64"] = out["fp64"]["ms_per_build"] / out["mixed"]["ms_per_build"]
    out["mixed"]["single_build_energy_error_eh"] = abs(0.5 * float((D * (Gs["mixed"] - Gs["fp64"])).sum().item()))
    # launch parameters of the mixed build chosen by the autotuner (fresh cache):
    # slicing, block size and persistent (work-queue) launches
    import tempfile
    from fock_gb300.tuning import autotune
    with tempfile.TemporaryDirectory() as td:
        tuned = autotune(ctx, D.data_ptr(), reps=2, cache_path=os.path.join(td, "tune.json"))
    t = _event_times(torch, stream, lambda: ctx.build_jk_device(D.data_ptr(), G.data_ptr()), steps, warmup, flush)
    ms_t = sum(t) / len(t)
    out["mixed_autotuned"] = {"ms_per_build": ms_t, "quartets_per_s": nq / (ms_t * 1e-3),
                              "speedup_vs_fp64": out["fp64"]["ms_per_build"] / ms_t,
                              "tuning": {k: tuned[k] for k in ("prims_per_slice", "prims_per_slice_fp32",
                                                               "block_threads", "persistent")}}
    ctx.close()
    if builds_only:
        return out
    # warm-up: a one-iteration SCF of the cluster pays the process's one-time costs
    # of the first large-basis SCF (cuSOLVER loading at n = 608, the atomic
    # densities of O and H in 6-31G*) outside the timed SCFs below
    with F.FockContext(atoms, precision=L.FOCK_PREC_FP64, guess=L.FOCK_GUESS_SAD, max_iters=1,
                       device=local) as wctx:
        wctx.scf(0)
    # mixed-precision SCF (final iterations FP64) and the nuclear gradient: analytic
    # derivative kernels for the s/p classes, finite-difference kernels for the d classes
    with F.FockContext(atoms, precision=L.FOCK_PREC_MIXED, guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY,
                       energy_mode=1, epsilon=1e-8, max_iters=100, level_shift=BATCH_LEVEL_SHIFT,
                       device=local) as sctx:
        t0 = time.perf_counter()
        rc, r, _, _, _ = sctx.scf(0)
        torch.cuda.synchronize()
        scf_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        g = sctx.energy_backward()
        grad_s = time.perf_counter() - t0
    out["scf_mixed"] = {"rc": rc, "wall_s": scf_s, "iterations": r.iterations, "energy": r.total_energy,
                        "level_shift_eh": BATCH_LEVEL_SHIFT, "guess": SCF_GUESS_NAME,
                        "energy_per_water": r.total_energy / 32,
                        "converged": bool(r.converged), "fock_builds": r.fock_builds, "fock_s": r.fock_seconds}
    with F.FockContext(atoms, precision=L.FOCK_PREC_FP64, guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY,
                       energy_mode=1, epsilon=1e-8, max_iters=100, level_shift=BATCH_LEVEL_SHIFT,
                       device=local) as fctx:
        t0 = time.perf_counter()
        rc64, r64, _, _, _ = fctx.scf(0)
        torch.cuda.synchronize()
        scf64_s = time.perf_counter() - t0
    out["scf_fp64"] = {"rc": rc64, "wall_s": scf64_s, "iterations": r64.iterations, "energy": r64.total_energy,
                       "converged": bool(r64.converged), "fock_builds": r64.fock_builds, "fock_s": r64.fock_seconds}
    out["scf_mixed"]["speedup_vs_fp64_scf"] = scf64_s / scf_s
    out["scf_mixed"]["abs_energy_error_vs_fp64_eh"] = abs(r.total_energy - r64.total_energy)
    out["gradient"] = {"wall_s": grad_s, "max_abs": float(np.abs(g).max()),
                       "net_force": float(np.abs(g.sum(axis=0)).max()), "components": int(g.size)}
    return out


def shard_balance_workload(torch, F, L, local, flush, steps=3, warmup=2, ks=(2, 4, 8)):
    """Row shards of the (H2O)32 / 6-31G* FP64 build (the multi-GPU split: rows
    r % k == rank, one all-reduce of G per build), measured on this one GPU:
    every shard's build time and quartet counts, run one after another.  The
    slowest shard bounds a k-GPU build; the all-reduce of the 608 x 608 G
    (2.96 MB) is not included."""
    from fock_gb300 import basis as B, molecules as M
    Zs, xyz = M.water_cluster(32, seed=0)
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    stream = torch.cuda.Stream()
    out = {"workload": "(H2O)32 seed 0, RHF/6-31G*, FP64 build, row shards r % k on one GPU"}
    D = G = None
    full_ms = None
    for k in (1,) + tuple(ks):
        shards = []
        for r in range(k):
            with F.FockContext(atoms, sign_convention=L.FOCK_SIGN_STANDARD, device=local, shard_index=r,
                               shard_count=k) as ctx:
                if D is None:
                    n = ctx.n
                    rng = np.random.default_rng(0)
                    Cm = rng.normal(size=(n, 160)) / np.sqrt(n)
                    D = torch.tensor(2.0 * Cm @ Cm.T, device="cuda")
                    G = torch.empty_like(D)
                ctx.set_stream(stream.cuda_stream)
                t = _event_times(torch, stream, lambda: ctx.build_jk_device(D.data_ptr(), G.data_ptr()), steps,
                                 warmup, flush)
                st = ctx.stats()
                shards.append({"ms": sum(t) / len(t), "shell_quartets": st["shell_quartets_fp64"],
                               "prim_quartets": st["prim_quartets_fp64"], "flops": st["flops_fp64"]})
        ms = [x["ms"] for x in shards]
        fl = [x["flops"] for x in shards]
        if k == 1:
            full_ms = ms[0]
            out["full_build_ms"] = full_ms
            continue
        out["k%d" % k] = {"shard_ms": [round(x, 3) for x in ms],
                          "max_over_mean_ms": max(ms) / (sum(ms) / k),
                          "max_over_mean_flops": max(fl) / (sum(fl) / k),
                          "shell_quartets": [x["shell_quartets"] for x in shards],
                          "projected_speedup": full_ms / max(ms)}
    return out


def octane_gradient_workload(torch, F, L, local):
    """n-octane C8H18 (seed 0, sigma 0.05 A), RHF/6-31G: FP64 SCF, then the
    nuclear gradient through fock_energy_backward (derivative ERIs contracted
    with the density on the fly + one-electron derivatives), wall-timed."""
    from fock_gb300 import basis as B, molecules as M
    Zs, xyz = M.octane(seed=0)
    atoms = B.build_atoms("6-31G", Zs, xyz)
    with F.FockContext(atoms, guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1,
                       max_iters=100, epsilon=1e-10, device=local) as ctx:
        t0 = time.perf_counter()
        rc, r, eps, Dm, Cm = ctx.scf(0)
        scf_s = time.perf_counter() - t0
        ctx.energy_backward()  # warm-up (plans the derivative launches)
        torch.cuda.synchronize()
        reps = []
        for _ in range(3):
            t0 = time.perf_counter()
            g = ctx.energy_backward()
            reps.append(time.perf_counter() - t0)
    return {"workload": "n-octane C8H18 seed 0, RHF/6-31G, 108 functions", "scf_s": scf_s, "scf_rc": rc,
            "energy": r.total_energy, "iterations": r.iterations, "gradient_s": min(reps),
            "max_abs_gradient": float(np.abs(g).max()), "net_force": float(np.abs(g.sum(axis=0)).max())}


def orbital_grid_workload(torch, F, L, local, atoms, C, nocc, opts, steps=3, warmup=2):
    """HOMO of benzene on the reference viewer's grid (200^3 voxels, box 20 bohr,
    |c| > 0.05), written to device memory; CUDA-event time per grid."""
    with F.FockContext(atoms, **opts) as ctx:
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
        homo = np.ascontiguousarray(C[:, nocc - 1])
        nvox = 200
        grid = torch.empty(nvox ** 3, dtype=torch.float32, device="cuda")
        for _ in range(warmup):
            ctx.orbital_grid_device(homo, grid.data_ptr(), nvox=nvox)
        ev = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.orbital_grid_device(homo, grid.data_ptr(), nvox=nvox)
            e1.record(stream)
            ev.append((e0, e1))
        stream.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ev)
        nsel = int((np.abs(homo) > 0.05).sum())
    return {"workload": "benzene HOMO on 200^3 voxels, box 20 bohr (volumetric viewer grid)",
            "ms_per_grid": ms, "voxels_per_s": nvox ** 3 / (ms * 1e-3), "functions_kept": nsel,
            "bytes_written": nvox ** 3 * 4}


def profile_classes(torch, lib, ctx, D, flush, reps=3):
    """Per-class launch times of one build, the classes launched one by one
    (fock_profile_build), averaged over reps builds: {"(ab|cd)[f32]": {...}}."""
    from fock_gb300 import _lib
    cap = 512
    arr = (_lib.LaunchProfile * cap)()
    per_class = {}
    for _ in range(reps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        np_ = lib.fock_profile_build(ctx.handle, C.c_void_p(D.data_ptr()), arr, cap)
        for i in range(min(np_, cap)):
            a = arr[i]
            key = "(%d%d|%d%d)%s" % (a.la, a.lb, a.lc, a.ld, "" if a.prec == 0 else "f32")
            d = per_class.setdefault(key, {"ms": 0.0, "flops": 0, "launches": 0, "prim_quartets": 0})
            d["ms"] += a.ms / reps
            d["flops"] += a.flops // reps
            d["launches"] += 1
            d["prim_quartets"] += a.prim_quartets // reps
    for d in per_class.values():
        d["launches"] //= reps
    return per_class


def parallelism(world):
    return "row shards (r %% %d) + NCCL all-reduce of G" % world if world > 1 else "single"


def run_reference_arm(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    value, cb = cpu_reference(args.steps, args.warmup)
    cb["value"] = value
    cb["unit"] = UNIT
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * WORKLOAD["unique_quartets"] / value,
            "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": dict(WORKLOAD, parallelism=parallelism(world)),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scf", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batch, (H2O)32 and gradient workloads")
    ap.add_argument("--only", choices=["benzene", "benzene_mixed", "batch", "water32", "water32_builds", "octane",
                                       "shards"],
                    help="run one side workload alone (profiling) and print its JSON")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import fock_gb300 as F
    from fock_gb300 import _lib as L
    if args.only:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        fn = {"benzene": lambda: benzene_builds(torch, F, L, local, flush, args.steps, args.warmup),
              "benzene_mixed": lambda: benzene_builds(torch, F, L, local, flush, args.steps, args.warmup,
                                                      L.FOCK_PREC_MIXED),
              "water32_builds": lambda: water32_workload(torch, F, L, local, flush, args.steps, args.warmup, True),
              "batch": lambda: batch_workload(torch, F, L, local, flush, args.steps, args.warmup),
              "water32": lambda: water32_workload(torch, F, L, local, flush, args.steps, args.warmup),
              "octane": lambda: octane_gradient_workload(torch, F, L, local),
              "shards": lambda: shard_balance_workload(torch, F, L, local, flush)}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return
    atoms = benzene_atoms()
    opts = dict(guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, device=local,
                sign_convention=L.FOCK_SIGN_STANDARD)
    extra = {}
    # one-time start-up (CUDA context, library tables, cuBLAS/cuSOLVER kernels) outside the SCF timings
    from fock_gb300 import basis as B, molecules as M
    F.try_scf(B.build_atoms("STO-3G", *M.water_sto3g()), 20, 1e-6, 0, **opts)
    # converged density (FP64 SCF) for the benchmark builds; SCF wall times
    t0 = time.perf_counter()
    r64 = F.try_scf(atoms, 100, 1e-9, 0, **opts)
    scf64_s = time.perf_counter() - t0
    rmx = None
    if not args.no_scf:
        t0 = time.perf_counter()
        rmx = F.try_scf(atoms, 100, 1e-9, 0, precision=L.FOCK_PREC_MIXED, **opts)
        scfmx_s = time.perf_counter() - t0
        extra["scf"] = {"guess": SCF_GUESS_NAME, "fp64_wall_s": scf64_s, "fp64_iterations": r64.iterations, "fp64_energy": r64.total_energy,
                        "fp64_fock_builds": r64.fock_builds, "fp64_fock_s": r64.fock_seconds,
                        "mixed_wall_s": scfmx_s, "mixed_iterations": rmx.iterations,
                        "mixed_energy": rmx.total_energy, "mixed_fock_s": rmx.fock_seconds,
                        "abs_energy_error_mixed_vs_fp64_eh": abs(rmx.total_energy - r64.total_energy)}
    # under torchrun every rank builds its row shard of the quartet plan (rows
    # r % world == rank) and one all-reduce of G per build completes it
    shard = dict(shard_index=rank, shard_count=world) if world > 1 else {}
    ctx = F.FockContext(atoms, **opts, **shard)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    n = ctx.n
    D = torch.tensor(r64.density_matrix, dtype=torch.float64, device="cuda")
    G = torch.empty((n, n), dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    nq = WORKLOAD["unique_quartets"]

    def one_build():
        ctx.build_jk_device(D.data_ptr(), G.data_ptr())
        if dist:
            dist.all_reduce(G)  # partial G of the row shards -> G (on the current stream)

    def timed_builds(k, w):
        with torch.cuda.stream(stream):
            for _ in range(w):
                one_build()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
            for e0, e1 in ev:
                flush.fill_(1.0)
                e0.record(stream)
                one_build()
                e1.record(stream)
        stream.synchronize()
        return [e0.elapsed_time(e1) for e0, e1 in ev]

    # ---- plain FP64 (headline) ----
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    clocks.start()
    times = timed_builds(args.steps, args.warmup)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = ctx.launch_count() - l0
    ms = sum(times) / len(times)
    ms_max = ms
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    value = nq / (ms_max * 1e-3)
    st = ctx.stats()

    # ---- per-launch profile -> dominant kernel roofline ----
    from fock_gb300 import _lib
    lib = _lib.lib()
    per_class = profile_classes(torch, lib, ctx, D, flush)
    total_ms = sum(d["ms"] for d in per_class.values())
    dom_key = max(per_class, key=lambda k: per_class[k]["ms"])
    dom = per_class[dom_key]
    fp64_peak_gflops = C.c_double()
    lib.fock_measure_fma_peak(local, 1, C.byref(fp64_peak_gflops))
    fp32_peak_gflops = C.c_double()
    lib.fock_measure_fma_peak(local, 0, C.byref(fp32_peak_gflops))
    achieved = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
    peak = fp64_peak_gflops.value / 1e3
    build_flops = st["flops_fp64"]
    # The class kernels of one build run concurrently from one CUDA graph (8
    # streams), so the unit timed live is the whole build: its algorithmic
    # flops over the CUDA-event time of the timed builds.  Per-class figures
    # come from fock_profile_build, which launches the classes one by one.
    build_achieved = build_flops / (ms * 1e-3) / 1e12
    roofline = {"bound": "fp64_pipe",
                "kernel": "eri_kernel class launches of one FP64 Fock build (one CUDA graph, %d launches)"
                          % st["launches_per_build"],
                "achieved": build_achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": build_achieved / peak if peak else None,
                # DRAM bytes of the six class kernels of one build, read from the ncu launch list of
                # `bench.py --only benzene` (cold caches, serialised launches); the warm concurrent
                # build reads its pair data and tables from L2
                "traffic": BUILD_DRAM_BYTES_NCU,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum summed over one build's class "
                                  "launches, from the launch list of `bench.py --only benzene` (cold caches, "
                                  "serialised launches), not measured in this run",
                "flops_per_build": build_flops,
                "peak_source": "measured FP64 FMA microbenchmark in this run (fock_measure_fma_peak); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "dominant_class": {"kernel": "eri_kernel %s" % dom_key, "achieved_serialised": achieved,
                                   "frac_serialised": achieved / peak if peak else None,
                                   "share_of_serialised_build": dom["ms"] / total_ms if total_ms else None},
                "fp32_peak_tflops": fp32_peak_gflops.value / 1e3,
                "per_class_ms_serialised": {k: round(v["ms"], 4) for k, v in sorted(per_class.items())}}

    # ---- mixed precision build (library default threshold) ----
    th = F.options().mixed_threshold
    ctx.set_precision(L.FOCK_PREC_MIXED, th)
    tmx = timed_builds(args.steps, args.warmup)
    ms_mx = sum(tmx) / len(tmx)
    stm = ctx.stats()
    Gm = G.clone()
    # per-class launch times of the mixed build (classes one by one): FP32 and FP64 shares
    pc_mx = profile_classes(torch, lib, ctx, D, flush)
    ctx.set_precision(L.FOCK_PREC_FP64, th)
    with torch.cuda.stream(stream):
        one_build()
    stream.synchronize()
    # energy of one mixed build at the converged density vs the FP64 build: 1/2 sum D (G_mixed - G_fp64)
    de_build = 0.5 * float((D * (Gm - G)).sum().item())
    # time-share roofline of the mixed build: FP32 flops at the FP32 peak plus FP64 flops at the FP64 peak
    mixed_frac = ((stm["flops_fp32"] / (fp32_peak_gflops.value * 1e9) + stm["flops_fp64"] / (peak * 1e12))
                  / (ms_mx * 1e-3)) if peak and fp32_peak_gflops.value else None
    mixed = {"value": nq / (ms_mx * 1e-3), "ms_per_step": ms_mx, "speedup_vs_fp64": ms / ms_mx,
             "per_class_ms_serialised": {k: round(v["ms"], 4) for k, v in sorted(pc_mx.items())},
             "roofline_time_share_frac": mixed_frac,
             "mixed_threshold": th, "fp32_shell_quartets": stm["shell_quartets_fp32"],
             "fp64_shell_quartets": stm["shell_quartets_fp64"],
             "max_abs_fock_error_vs_fp64": float((Gm - G).abs().max().item()),
             "single_build_energy_error_eh": abs(de_build)}
    if rmx is not None:
        mixed["abs_energy_error_vs_fp64_eh"] = abs(rmx.total_energy - r64.total_energy)
    # error per ERI of the FP32 kernels: the benzene tensor with every quartet in FP32
    if rank == 0:
        t64 = F.ElectronTensor.from_basis(atoms, device=local).data
        t32 = F.ElectronTensor.from_basis(atoms, device=local, precision=L.FOCK_PREC_MIXED,
                                          mixed_threshold=1e30).data
        err = np.abs(t32 - t64)
        big = np.abs(t64) > 1e-3
        mixed["fp32_eri_error"] = {"max_abs": float(err.max()), "rms_abs": float(np.sqrt((err ** 2).mean())),
                                   "max_rel_for_abs_above_1e-3": float((err[big] / np.abs(t64[big])).max()),
                                   "integrals": int(t64.size)}
        del t64, t32, err

    # ---- e2e through the C ABI with host buffers ----
    Dh = np.ascontiguousarray(r64.density_matrix)
    ctx.set_stream(0)

    def e2e_build():
        Gh = ctx.build_jk(Dh)
        if dist:  # the partial G of this rank's shard, summed over the ranks on the device
            Gt = torch.from_numpy(Gh).cuda()
            dist.all_reduce(Gt)
            Gh = Gt.cpu().numpy()
        return Gh

    for _ in range(args.warmup):
        e2e_build()
    te = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        e2e_build()
        te.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(te)
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": nq / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * n * 8 * (2 if dist else 1),
           "d2h_bytes_per_step": n * n * 8 * (2 if dist else 1),
           "ms_per_step": e2e_s * 1e3, "api": "fock_build_jk (host D in, host G out)" +
           (" + all-reduce of G over the ranks" if dist else "")}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, cb = cpu_reference(1, 0)
            cb["value"] = v
            cb["unit"] = UNIT
            cpu = cb
        except Exception as ex:  # baseline is reported, never fatal
            cpu = {"value": None, "error": str(ex)[:200]}

    if rank == 0 and not args.no_extra:
        extra["workloads"] = {}
        for key, fn in (("batch_512_water_clusters_631g", lambda: batch_workload(torch, F, L, local, flush)),
                        ("water32_631gs", lambda: water32_workload(torch, F, L, local, flush)),
                        ("octane_631g_gradient", lambda: octane_gradient_workload(torch, F, L, local)),
                        ("shard_balance_water32", lambda: shard_balance_workload(torch, F, L, local, flush)),
                        ("orbital_grid_benzene_homo", lambda: orbital_grid_workload(
                            torch, F, L, local, atoms, r64.coefficient_matrix, r64.n_electrons // 2, opts))):
            try:
                extra["workloads"][key] = fn()
            except Exception as ex:  # reported beside the headline, never fatal
                extra["workloads"][key] = {"error": repr(ex)[:300]}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max,
                # spread of this rank's timed steps (ms_per_step is their mean)
                "ms_per_step_median": statistics.median(times), "ms_per_step_min": min(times),
                "higher_is_better": True,
                "scaling": "strong" if world > 1 else "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(WORKLOAD, parallelism=parallelism(world)),
                "clocks": clk, "gpu_launches": launches, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "mixed": mixed, "stats": {k: st[k] for k in ("shell_quartets_fp64", "prim_quartets_fp64",
                                                               "shell_quartets_screened", "launches_per_build")}}
        line.update(extra)
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
