"""Generate the committed golden fixtures under tests/golden/.

Run once where the reference sources and mpmath are present:
  FOCK_REFERENCE_ROOT=<fock-rs checkout> python tests/golden/make_golden.py [--lut-only]

Fixtures
  fock-rs_gb300/data/boys_ref_lut.json
                       the reference's 200 stored F_10 values (boys/src/lut.rs),
                       read by the library's reference-compatible mode and by
                       the oracle (--lut-only writes this file alone).
  boys_mpmath.json     F_n(t) at 30 digits (mpmath), n = 0..12, t on a log grid
                       plus points next to the Boys table nodes.
  h2o_sto3g_ref.json   H2O / STO-3G (the water workload), computed by a pure-
                       Python restatement of the reference written independently
                       of oracle/fock_oracle.cpp:
                         boys            boys/src/lib.rs:58-81 with the LUT
                                         values read from boys/src/lut.rs
                         hermite_expansion basis/src/utils.rs:33-50
                         coulomb_auxiliary basis/src/utils.rs:73-106 (x branch
                                         as written there, and corrected)
                         norm            basis/src/primitives.rs:19-27
                         ERIs / S / T / V basis/src/contracted_gaussian.rs
                       It stores all 406 unique ERIs in the reference's sign
                       convention for the reference behaviour ("refcompat":
                       LUT Boys + x-branch as written) and exact behaviour
                       (mpmath Boys + corrected recursion), S/T/V, and the RHF
                       energy of scf/src/lib.rs:73-258 (GWH guess, DIIS 16/5,
                       commutator < 1e-6) for both.
"""
import json
import math
import os
import re
import sys

import mpmath
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "fock-rs_gb300"))
from fock_gb300 import basis as B  # noqa: E402
from fock_gb300 import molecules as M  # noqa: E402

mpmath.mp.dps = 40


def boys_mp(n, t):
    t = mpmath.mpf(t)
    if t == 0:
        return mpmath.mpf(1) / (2 * n + 1)
    # F_n(t) = gamma(n+1/2) P(n+1/2, t) / (2 t^(n+1/2))
    return mpmath.gammainc(n + 0.5, 0, t) / (2 * t ** (n + 0.5))


def make_boys():
    ts = sorted(set([0.0] + [float(x) for x in np.logspace(-12, 2.3, 220)] +
                    [k / 16.0 + d for k in range(0, 1025, 37) for d in (-1 / 33.0, 0.0, 1 / 33.0) if k / 16.0 + d > 0] +
                    [29.9, 30.0, 30.1, 63.99, 64.0, 64.01, 120.0]))
    rows = []
    for t in ts:
        rows.append([t] + [float(boys_mp(n, t)) for n in range(13)])
    return {"orders": 13, "rows": rows, "source": "mpmath gammainc, 40 digits"}


# ---------------- pure-Python restatement of the reference ----------------

class Ref:
    def __init__(self, lut, exact):
        self.lut = lut
        self.exact = exact

    def boys(self, t, n):
        if self.exact:
            return float(boys_mp(n, t))
        if abs(t) < 1e-16:
            return 1.0 / (2 * n + 1)
        if abs(t) >= 30.0:
            arg = max(2 * n - 1, 0)
            df = 1
            k = 2 - arg % 2 if arg > 0 else 1
            while arg > 0 and k <= arg:
                df *= k
                k += 2
            return df * (1.0 / 2.0 ** (n + 1)) * math.sqrt(math.pi * t ** (-2 * n - 1))
        N = 200
        index_f = N * t / 30.0
        lower, upper = math.floor(index_f), math.ceil(index_f)
        int_t = index_f - lower
        cur = int_t * self.lut[min(int(upper), N - 1)] + (1.0 - int_t) * self.lut[int(lower)]
        e = math.exp(-t)
        cn = 10
        while cn > n:
            cur = (2.0 * t * cur + e) / (2 * cn - 1)
            cn -= 1
        return cur

    @staticmethod
    def hermite(i, j, t, dist, a, b):
        p = a + b
        q = a * b / p
        if t < 0 or t > i + j:
            return 0.0
        if i == j == t == 0:
            return math.exp(-q * dist * dist)
        if j == 0:
            return ((1.0 / (2.0 * p)) * Ref.hermite(i - 1, j, t - 1, dist, a, b)
                    - (q * dist / a) * Ref.hermite(i - 1, j, t, dist, a, b)
                    + (t + 1) * Ref.hermite(i - 1, j, t + 1, dist, a, b))
        return ((1.0 / (2.0 * p)) * Ref.hermite(i, j - 1, t - 1, dist, a, b)
                + (q * dist / b) * Ref.hermite(i, j - 1, t, dist, a, b)
                + (t + 1) * Ref.hermite(i, j - 1, t + 1, dist, a, b))

    def coulomb(self, t, u, v, n, p, d, r2):
        if t == u == v == 0:
            return (-2.0 * p) ** n * self.boys(p * r2, n)
        if t == 0 and u == 0:
            return d[2] * self.coulomb(t, u, v - 1, n + 1, p, d, r2) + (
                (v - 1) * self.coulomb(t, u, v - 2, n + 1, p, d, r2) if v > 1 else 0.0)
        if t == 0:
            return d[1] * self.coulomb(t, u - 1, v, n + 1, p, d, r2) + (
                (u - 1) * self.coulomb(t, u - 2, v, n + 1, p, d, r2) if u > 1 else 0.0)
        fac = (t - 1) if self.exact else 1.0
        return d[0] * self.coulomb(t - 1, u, v, n + 1, p, d, r2) + (
            fac * self.coulomb(t - 2, u, v, n + 1, p, d, r2) if t > 1 else 0.0)


def norm(ang, alpha):
    def prod(lo, hi):
        r = 1
        for k in range(lo, hi + 1):
            r *= k
        return r
    den = prod(ang[0] + 1, 2 * ang[0]) * prod(ang[1] + 1, 2 * ang[1]) * prod(ang[2] + 1, 2 * ang[2])
    return math.sqrt(math.sqrt((2.0 / math.pi * alpha) ** 3)) * math.sqrt((8.0 * alpha) ** sum(ang) / den)


def functions(atoms):
    fs = []
    for sh in B.shells_of(atoms):
        for comp in B.cartesian_components(sh.l):
            prims = [(comp, float(e), float(c) * norm(comp, float(e))) for e, c in zip(sh.exps, sh.coefs)]
            fs.append((np.array(sh.center, dtype=float), prims))
    return fs


def prim_eri(R, pr, dab, dcd, cdiff, r2):
    (A, a, _), (Bv, b, _), (Cv, c, _), (Dv, d, _) = pr
    p, q = a + b, c + d
    alpha = p * q / (p + q)
    s = 0.0
    for t1 in range(A[0] + Bv[0] + 1):
        e1 = Ref.hermite(A[0], Bv[0], t1, dab[0], a, b)
        for u1 in range(A[1] + Bv[1] + 1):
            e2 = Ref.hermite(A[1], Bv[1], u1, dab[1], a, b)
            for v1 in range(A[2] + Bv[2] + 1):
                e3 = Ref.hermite(A[2], Bv[2], v1, dab[2], a, b)
                for t2 in range(Cv[0] + Dv[0] + 1):
                    e4 = Ref.hermite(Cv[0], Dv[0], t2, dcd[0], c, d)
                    for u2 in range(Cv[1] + Dv[1] + 1):
                        e5 = Ref.hermite(Cv[1], Dv[1], u2, dcd[1], c, d)
                        for v2 in range(Cv[2] + Dv[2] + 1):
                            e6 = Ref.hermite(Cv[2], Dv[2], v2, dcd[2], c, d)
                            s += (e1 * e2 * e3 * e4 * e5 * e6 * R.coulomb(t1 + t2, u1 + u2, v1 + v2, 0, alpha, cdiff, r2)
                                  * (1.0 if (t2 + u2 + v2) % 2 == 0 else -1.0))
    return 2.0 * math.sqrt(math.pi ** 5) * (1.0 / (p * q * math.sqrt(p + q))) * s


def eri(R, fa, fb, fc, fd):
    dab = fb[0] - fa[0]
    dcd = fd[0] - fc[0]
    tot = 0.0
    for pa in fa[1]:
        for pb in fb[1]:
            pab = (pa[1] * fa[0] + pb[1] * fb[0]) / (pa[1] + pb[1])
            for pc in fc[1]:
                for pd in fd[1]:
                    pcd = (pc[1] * fc[0] + pd[1] * fd[0]) / (pc[1] + pd[1])
                    cdiff = pcd - pab
                    r2 = float(cdiff @ cdiff)
                    tot += pa[2] * pb[2] * pc[2] * pd[2] * prim_eri(R, (pa, pb, pc, pd), dab, dcd, cdiff, r2)
    return tot


def one_electron(R, fs, atoms):
    n = len(fs)
    S, T, V = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))

    def ov(A, a, Bv, b, diff):
        if min(A) < 0 or min(Bv) < 0:
            return 0.0
        return (Ref.hermite(A[0], Bv[0], 0, diff[0], a, b) * Ref.hermite(A[1], Bv[1], 0, diff[1], a, b)
                * Ref.hermite(A[2], Bv[2], 0, diff[2], a, b) * math.sqrt((math.pi / (a + b)) ** 3))

    for i in range(n):
        for j in range(i, n):
            (ca, pa_), (cb, pb_) = fs[i], fs[j]
            diff = cb - ca
            s = t = v = 0.0
            for (A, a, xa) in pa_:
                for (Bv, b, xb) in pb_:
                    s += xa * xb * ov(A, a, Bv, b, diff)
                    l2, m2, n2 = Bv

                    def st(di, dj, dk):
                        return ov(A, a, (Bv[0] + di, Bv[1] + dj, Bv[2] + dk), b, diff)
                    term0 = b * (2 * (l2 + m2 + n2) + 3) * ov(A, a, Bv, b, diff)
                    term1 = -2.0 * b * b * (st(2, 0, 0) + st(0, 2, 0) + st(0, 0, 2))
                    term2 = -0.5 * (l2 * (l2 - 1) * st(-2, 0, 0) + m2 * (m2 - 1) * st(0, -2, 0) + n2 * (n2 - 1) * st(0, 0, -2))
                    t += xa * xb * (term0 + term1 + term2)
                    p = a + b
                    P = (a * ca + b * cb) / p
                    for at in atoms:
                        dcp = at.position - P
                        r2 = float(dcp @ dcp)
                        acc = 0.0
                        for tt in range(A[0] + Bv[0] + 1):
                            for u in range(A[1] + Bv[1] + 1):
                                for w in range(A[2] + Bv[2] + 1):
                                    acc += (Ref.hermite(A[0], Bv[0], tt, diff[0], a, b)
                                            * Ref.hermite(A[1], Bv[1], u, diff[1], a, b)
                                            * Ref.hermite(A[2], Bv[2], w, diff[2], a, b)
                                            * R.coulomb(tt, u, w, 0, p, dcp, r2))
                        v += xa * xb * (-at.Z * 2.0 * math.pi / p * acc)
            S[i, j] = S[j, i] = s
            T[i, j] = T[j, i] = t
            V[i, j] = V[j, i] = v
    return S, T, V


def scf_reference(S, H, eri4, nel, max_iters=100, eps=1e-6):
    """scf/src/lib.rs:73-258 in numpy (GWH guess, DIIS 16/5, commutator)."""
    n = S.shape[0]
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    Hg = 0.875 * S * (np.diag(H)[:, None] + np.diag(H)[None, :])

    def dens(F):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        Cm = X @ Cp
        return 2.0 * Cm[:, :nel // 2] @ Cm[:, :nel // 2].T
    D = dens(Hg)
    focks, errs = [], []
    for it in range(max_iters + 1):
        J = np.einsum("ijkl,kl->ij", eri4, D)
        K = np.einsum("ikjl,kl->ij", eri4, D)
        G = J - 0.5 * K
        F = H + G
        E = F @ D @ S - S @ D @ F
        err = np.abs(E).max()
        errs.append(E)
        focks.append(F)
        if len(errs) > 16:
            errs.pop(0)
            focks.pop(0)
        Fd = focks[-1]
        if len(focks) >= 5:
            m = len(errs)
            Bm = np.zeros((m + 1, m + 1))
            for i in range(m):
                for j in range(m):
                    Bm[i, j] = np.sum(errs[i] * errs[j])
            Bm[m, :m] = -1.0
            Bm[:m, m] = -1.0
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            c = np.linalg.solve(Bm, rhs)
            Fd = sum(c[i] * focks[i] for i in range(m))
        Dn = dens(Fd)
        e_el = 0.5 * np.sum(Dn * (2.0 * H + G))
        if err < eps or it == max_iters:
            return e_el, it
        D = Dn
    return None


def read_lut(ref_root):
    """The reference's stored F_10(0.15 k), k < 200 (boys/src/lut.rs), as written there."""
    src = open(os.path.join(ref_root, "boys/src/lut.rs")).read()
    lut = [float(x) for x in re.findall(r"[-+0-9.eE]+(?=,)", src.split("=", 1)[1])]
    assert len(lut) == 200
    return lut


def write_lut(ref_root):
    """Data file shared by the library's reference-compatible mode and the oracle."""
    dst = os.path.join(os.path.dirname(os.path.dirname(HERE)), "fock-rs_gb300", "data", "boys_ref_lut.json")
    with open(dst, "w") as f:
        json.dump({"source": "boys/src/lut.rs of fock-rs (F_10(0.15 k), k = 0..199, as stored there)",
                   "dt": 0.15, "order": 10, "values": read_lut(ref_root)}, f, indent=0)
    print("wrote", dst)


def make_h2o(ref_root):
    lut = read_lut(ref_root)
    Zs, xyz = M.water_sto3g()
    atoms = B.build_atoms("STO-3G", Zs, xyz)
    fs = functions(atoms)
    n = len(fs)
    out = {"n": n, "coords_bohr": xyz.tolist(), "Z": Zs, "basis": "STO-3G",
           "sign_convention": "reference (A-r)^l", "quartets": [], "modes": {}}
    quartets = [(i, j, k, l) for i in range(n) for j in range(i + 1) for k in range(n) for l in range(k + 1)
                if i * (i + 1) // 2 + j >= k * (k + 1) // 2 + l]
    out["quartets"] = quartets
    nel = sum(Zs)
    for mode, R in (("refcompat", Ref(lut, exact=False)), ("exact", Ref(lut, exact=True))):
        vals = [eri(R, fs[i], fs[j], fs[k], fs[l]) for (i, j, k, l) in quartets]
        S, T, V = one_electron(R, fs, atoms)
        eri4 = np.zeros((n, n, n, n))
        diag = {}
        for (i, j, k, l), v in zip(quartets, vals):
            if (i, j) == (k, l):
                diag[(i, j)] = v
        for (i, j, k, l), v in zip(quartets, vals):
            if mode == "refcompat" and (i, j) != (k, l) and not (math.sqrt(diag[(i, j)] * diag[(k, l)]) > 1e-6):
                v = 0.0
            for (a, b, c, d) in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k), (k, l, i, j), (l, k, i, j),
                                 (k, l, j, i), (l, k, j, i)):
                eri4[a, b, c, d] = v
        vnn = 0.0
        for a in range(len(atoms)):
            for b in range(a + 1, len(atoms)):
                vnn += atoms[a].Z * atoms[b].Z / np.linalg.norm(atoms[a].position - atoms[b].position)
        e_el, it = scf_reference(S, T + V, eri4, nel)
        out["modes"][mode] = {"eri": vals, "S": S.tolist(), "T": T.tolist(), "V": V.tolist(),
                              "electronic_energy": e_el, "total_energy": e_el + vnn, "iterations": it,
                              "nuclear_repulsion": vnn}
        print(mode, "E =", e_el + vnn, "iters", it)
    return out


def main(ref_root, lut_only=False):
    write_lut(ref_root)
    if lut_only:
        return
    with open(os.path.join(HERE, "boys_mpmath.json"), "w") as f:
        json.dump(make_boys(), f)
    with open(os.path.join(HERE, "h2o_sto3g_ref.json"), "w") as f:
        json.dump(make_h2o(ref_root), f)


if __name__ == "__main__":
    root = os.environ.get("FOCK_REFERENCE_ROOT")
    if not root:
        sys.exit("set FOCK_REFERENCE_ROOT to the root of a fock-rs checkout")
    main(root, lut_only="--lut-only" in sys.argv[1:])
