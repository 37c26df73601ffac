"""Generate the per-class ERI recurrences (Obara-Saika VRR + Head-Gordon-Pople HRR).

For a shell-quartet class (la lb | lc ld) with la >= lb, lc >= ld this emits a
struct ``Cls_<la>_<lb>_<lc>_<ld>`` with two device functions:

  vrr<R>(F, PA, WP, QC, WQ, o2p, o2q, o2pq, rp, rq, acc)
      builds the primitive integrals [e0|f0]^(0) for |e| in [la, la+lb],
      |f| in [lc, lc+ld] from the scaled Boys values F[m] = pref * F_m(T) and
      adds them into the contracted accumulator ``acc`` (row-major [e][f]);
  hrr<R>(acc, AB, CD, out)
      transfers angular momentum to b and d on the contracted values:
      (a, b+1_i| = (a+1_i, b| + AB_i (a b|,  AB = A - B, and the same on the
      ket with CD, writing out[((ia*NB + ib)*NC + ic)*ND + id].

Recurrences (textbook (r-A)^l convention, W = (pP+qQ)/(p+q), rho = pq/(p+q)):
  [e+1_i|f]^m = PA_i [e|f]^m + WP_i [e|f]^{m+1}
                + e_i/(2p) ([e-1_i|f]^m - rho/p [e-1_i|f]^{m+1})
                + f_i/(2(p+q)) [e|f-1_i]^{m+1}
  [e|f+1_i]^m = QC_i [e|f]^m + WQ_i [e|f]^{m+1}
                + f_i/(2q) ([e|f-1_i]^m - rho/q [e|f-1_i]^{m+1})
                + e_i/(2(p+q)) [e-1_i|f]^{m+1}
Cartesian components are in the reference's order (x outer, y, z inner,
ascending), i.e. p = (z, y, x), so the output index maps straight onto
basis-function offsets.

The generator also counts floating-point operations (an FMA counts as 2) per
primitive quartet (VRR) and per contracted quartet (HRR); these counts feed
the roofline model written to ``roofline_model.json``.

Usage: python gen_eri.py <outdir> <lmax>
"""
import json
import os
import sys


def comps(l):
    return [(x, y, z) for x in range(l + 1) for y in range(l + 1) for z in range(l + 1) if x + y + z == l]


def ncart(l):
    return (l + 1) * (l + 2) // 2


def add(v, i, d):
    v = list(v)
    v[i] += d
    return tuple(v)


def nm(t):
    return "%d%d%d" % t


class Emitter:
    def __init__(self):
        self.lines = []
        self.flops = 0


def pick_axis(v):
    # axis with the largest component (ties: x before y before z)
    best = max(range(3), key=lambda i: (v[i], -i))
    return best


def gen_vrr(la, lb, lc, ld):
    L = la + lb + lc + ld
    E = Emitter()
    memo = {}
    consts = set()

    def const(kind, k):
        name = "%s_%d" % (kind, k)
        if name not in consts:
            consts.add(name)
            E.lines.append("    const R %s = R(%d) * %s;" % (name, k, kind))
            E.flops += 1
        return name

    def get(e, f, m):
        if min(e) < 0 or min(f) < 0:
            return None
        key = (e, f, m)
        if key in memo:
            return memo[key]
        if sum(e) == 0 and sum(f) == 0:
            memo[key] = "F[%d]" % m
            return memo[key]
        name = "v%s_%s_%d" % (nm(e), nm(f), m)
        terms = []
        if sum(f) > 0:
            i = pick_axis(f)
            f1 = add(f, i, -1)
            a = get(e, f1, m)
            b = get(e, f1, m + 1)
            expr = "QC[%d] * %s + WQ[%d] * %s" % (i, a, i, b)
            fl = 3
            f2 = add(f1, i, -1)
            if f1[i] > 0:
                c = get(e, f2, m)
                d = get(e, f2, m + 1)
                k = const("o2q", f1[i])
                expr += " + %s * (%s - rq * %s)" % (k, c, d)
                fl += 4
            if e[i] > 0:
                g = get(add(e, i, -1), f1, m + 1)
                k = const("o2pq", e[i])
                expr += " + %s * %s" % (k, g)
                fl += 2
        else:
            i = pick_axis(e)
            e1 = add(e, i, -1)
            a = get(e1, f, m)
            b = get(e1, f, m + 1)
            expr = "PA[%d] * %s + WP[%d] * %s" % (i, a, i, b)
            fl = 3
            e2 = add(e1, i, -1)
            if e1[i] > 0:
                c = get(e2, f, m)
                d = get(e2, f, m + 1)
                k = const("o2p", e1[i])
                expr += " + %s * (%s - rp * %s)" % (k, c, d)
                fl += 4
        E.lines.append("    const R %s = %s;" % (name, expr))
        E.flops += fl
        memo[key] = name
        return name

    es = [c for l in range(la, la + lb + 1) for c in comps(l)]
    fs = [c for l in range(lc, lc + ld + 1) for c in comps(l)]
    nf = len(fs)
    acc_lines = []
    for ie, e in enumerate(es):
        for jf, f in enumerate(fs):
            v = get(e, f, 0)
            acc_lines.append("    acc[%d] += %s;" % (ie * nf + jf, v))
            E.flops += 1
    E.lines.extend(acc_lines)
    return E, len(es), nf, L


def gen_hrr(la, lb, lc, ld):
    """Emit HRR from acc[e][f] to out[a][b][c][d]."""
    E = Emitter()
    es = [c for l in range(la, la + lb + 1) for c in comps(l)]
    fs = [c for l in range(lc, lc + ld + 1) for c in comps(l)]
    eidx = {c: i for i, c in enumerate(es)}
    fidx = {c: i for i, c in enumerate(fs)}
    nf = len(fs)
    A, B, Cc, D = comps(la), comps(lb), comps(lc), comps(ld)
    # bra transfer for every f: (a b | f)
    bra_memo = {}

    def bra(a, b, f):
        key = (a, b, f)
        if key in bra_memo:
            return bra_memo[key]
        if sum(b) == 0:
            r = "acc[%d]" % (eidx[a] * nf + fidx[f])
            bra_memo[key] = r
            return r
        i = pick_axis(b)
        b1 = add(b, i, -1)
        x = bra(add(a, i, 1), b1, f)
        y = bra(a, b1, f)
        name = "h%s%s_%s" % (nm(a), nm(b), nm(f))
        E.lines.append("    const R %s = %s + AB[%d] * %s;" % (name, x, i, y))
        E.flops += 2
        bra_memo[key] = name
        return name

    ket_memo = {}

    def ket(a, b, c, d):
        key = (a, b, c, d)
        if key in ket_memo:
            return ket_memo[key]
        if sum(d) == 0:
            r = bra(a, b, c)
            ket_memo[key] = r
            return r
        i = pick_axis(d)
        d1 = add(d, i, -1)
        x = ket(a, b, add(c, i, 1), d1)
        y = ket(a, b, c, d1)
        name = "k%s%s%s%s" % (nm(a), nm(b), nm(c), nm(d))
        E.lines.append("    const R %s = %s + CD[%d] * %s;" % (name, x, i, y))
        E.flops += 2
        ket_memo[key] = name
        return name

    NB, NC, ND = len(B), len(Cc), len(D)
    for ia, a in enumerate(A):
        for ib, b in enumerate(B):
            for ic, c in enumerate(Cc):
                for id_, d in enumerate(D):
                    v = ket(a, b, c, d)
                    E.lines.append("    out[%d] = %s;" % (((ia * NB + ib) * NC + ic) * ND + id_, v))
    return E


def pair_classes(lmax):
    return [(a, b) for a in range(lmax + 1) for b in range(a + 1)]


def quartet_classes(lmax):
    pcs = pair_classes(lmax)
    out = []
    for i, x in enumerate(pcs):
        for y in pcs[: i + 1]:
            out.append(x + y)
    return out


def main(outdir, lmax):
    os.makedirs(outdir, exist_ok=True)
    classes = quartet_classes(lmax)
    model = {}
    hdr = ["// Generated by gen_eri.py: Obara-Saika VRR + HGP HRR per class. Do not edit.",
           "#pragma once", ""]
    for (la, lb, lc, ld) in classes:
        V, ne, nf, L = gen_vrr(la, lb, lc, ld)
        H = gen_hrr(la, lb, lc, ld)
        name = "Cls_%d_%d_%d_%d" % (la, lb, lc, ld)
        hdr.append("struct %s {" % name)
        hdr.append("  static constexpr int LA = %d, LB = %d, LC = %d, LD = %d, L = %d;" % (la, lb, lc, ld, L))
        hdr.append("  static constexpr int NE = %d, NF = %d;" % (ne, nf))
        hdr.append("  static constexpr int NA = %d, NB = %d, NC = %d, ND = %d;" % (ncart(la), ncart(lb), ncart(lc), ncart(ld)))
        hdr.append("  template <typename R>")
        hdr.append("  __device__ __forceinline__ static void vrr(const R* __restrict__ F, const R* PA, const R* WP, const R* QC, const R* WQ,")
        hdr.append("                                             R o2p, R o2q, R o2pq, R rp, R rq, R* acc) {")
        hdr.append("    (void)PA; (void)WP; (void)QC; (void)WQ; (void)o2p; (void)o2q; (void)o2pq; (void)rp; (void)rq;")
        hdr.extend(V.lines)
        hdr.append("  }")
        hdr.append("  template <typename R>")
        hdr.append("  __device__ __forceinline__ static void hrr(const R* __restrict__ acc, const R* AB, const R* CD, R* out) {")
        hdr.append("    (void)AB; (void)CD;")
        hdr.extend(H.lines)
        hdr.append("  }")
        hdr.append("};")
        hdr.append("")
        model["(%d%d|%d%d)" % (la, lb, lc, ld)] = {
            "L": L, "vrr_flops_per_prim_quartet": V.flops, "hrr_flops_per_quartet": H.flops,
            "n_eri_per_quartet": ncart(la) * ncart(lb) * ncart(lc) * ncart(ld),
        }
    with open(os.path.join(outdir, "eri_classes.cuh"), "w") as f:
        f.write("\n".join(hdr) + "\n")
    # one instantiation unit per class so nvcc can compile them in parallel
    names = []
    for (la, lb, lc, ld) in classes:
        name = "Cls_%d_%d_%d_%d" % (la, lb, lc, ld)
        names.append(name)
        with open(os.path.join(outdir, "inst_%d%d%d%d.cu" % (la, lb, lc, ld)), "w") as f:
            f.write('// Generated by gen_eri.py. Do not edit.\n#include "../eri_kernel.cuh"\n')
            f.write("namespace fockgb {\n")
            f.write("cudaError_t launch_%s(const ClassLaunch& cl, const EriArgs& a, int mode, int prec, cudaStream_t s) {\n" % name)
            f.write("  return launch_class<%s>(cl, a, mode, prec, s);\n}\n" % name)
            f.write("}  // namespace fockgb\n")
    with open(os.path.join(outdir, "dispatch.cuh"), "w") as f:
        f.write("// Generated by gen_eri.py. Do not edit.\n#pragma once\nnamespace fockgb {\n")
        for n in names:
            f.write("cudaError_t launch_%s(const ClassLaunch&, const EriArgs&, int, int, cudaStream_t);\n" % n)
        f.write("inline cudaError_t launch_eri_class(int la, int lb, int lc, int ld, const ClassLaunch& cl, const EriArgs& a, int mode, int prec, cudaStream_t s) {\n")
        f.write("  int key = ((la * 8 + lb) * 8 + lc) * 8 + ld;\n  switch (key) {\n")
        for (la, lb, lc, ld), n in zip(classes, names):
            f.write("    case %d: return launch_%s(cl, a, mode, prec, s);\n" % (((la * 8 + lb) * 8 + lc) * 8 + ld, n))
        f.write("    default: return cudaErrorInvalidValue;\n  }\n}\n")
        f.write("// flops of the generated recurrences: VRR per primitive quartet, HRR per contracted quartet\n")
        f.write("inline int generated_class_flops(int la, int lb, int lc, int ld, int* hrr, int* neri) {\n")
        f.write("  int key = ((la * 8 + lb) * 8 + lc) * 8 + ld;\n  switch (key) {\n")
        for (la, lb, lc, ld) in classes:
            m = model["(%d%d|%d%d)" % (la, lb, lc, ld)]
            f.write("    case %d: *hrr = %d; *neri = %d; return %d;\n" % (
                ((la * 8 + lb) * 8 + lc) * 8 + ld, m["hrr_flops_per_quartet"], m["n_eri_per_quartet"],
                m["vrr_flops_per_prim_quartet"]))
        f.write("    default: *hrr = 0; *neri = 0; return 0;\n  }\n}\n")
        f.write("constexpr int kGeneratedLmax = %d;\n" % lmax)
        f.write("}  // namespace fockgb\n")
    with open(os.path.join(outdir, "roofline_model.json"), "w") as f:
        json.dump(model, f, indent=1, sort_keys=True)
    return classes


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 2)
