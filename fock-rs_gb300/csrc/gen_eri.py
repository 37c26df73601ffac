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
import re
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

    terms_of = {}  # name -> [(coefficient, operand)], value = sum of coefficient * operand

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
        if sum(f) > 0:
            i = pick_axis(f)
            f1 = add(f, i, -1)
            a = get(e, f1, m)
            b = get(e, f1, m + 1)
            terms = [("QC[%d]" % i, a), ("WQ[%d]" % i, b)]
            fl = 3
            f2 = add(f1, i, -1)
            if f1[i] > 0:
                c = get(e, f2, m)
                d = get(e, f2, m + 1)
                k = const("o2q", f1[i])
                terms.append((k, "(%s - rq * %s)" % (c, d)))
                fl += 4
            if e[i] > 0:
                g = get(add(e, i, -1), f1, m + 1)
                k = const("o2pq", e[i])
                terms.append((k, g))
                fl += 2
        else:
            i = pick_axis(e)
            e1 = add(e, i, -1)
            a = get(e1, f, m)
            b = get(e1, f, m + 1)
            terms = [("PA[%d]" % i, a), ("WP[%d]" % i, b)]
            fl = 3
            e2 = add(e1, i, -1)
            if e1[i] > 0:
                c = get(e2, f, m)
                d = get(e2, f, m + 1)
                k = const("o2p", e1[i])
                terms.append((k, "(%s - rp * %s)" % (c, d)))
                fl += 4
        E.lines.append("    const R %s = %s;" % (name, " + ".join("%s * %s" % t for t in terms)))
        terms_of[name] = terms
        E.flops += fl
        memo[key] = name
        return name

    es = [c for l in range(la, la + lb + 1) for c in comps(l)]
    fs = [c for l in range(lc, lc + ld + 1) for c in comps(l)]
    nf = len(fs)
    targets = []
    for ie, e in enumerate(es):
        for jf, f in enumerate(fs):
            targets.append((ie * nf + jf, get(e, f, 0)))
            E.flops += 1
    # A target used by no other recurrence line is accumulated straight into
    # acc by a chain of FMAs (acc = fma(c_k, x_k, acc)) instead of being formed
    # and then added: one FP64 instruction less per contracted component.
    body = "\n".join(E.lines)
    acc_lines = []
    for j, v in targets:
        fused = v in terms_of and len(re.findall(r"\b%s\b" % v, body)) == 1
        if fused:
            E.lines = [ln for ln in E.lines if not ln.startswith("    const R %s = " % v)]
            for cf, op in terms_of[v]:
                acc_lines.append("    acc[%d] = fma(%s, %s, acc[%d]);" % (j, cf, op, j))
        else:
            acc_lines.append("    acc[%d] += %s;" % (j, v))
    if L == 1:
        # (ps|ss): WP_i F_1 = PQ_i (-rp F_1); one multiply instead of forming WP (three)
        acc_lines = [ln.replace("fma(WP[", "fma(PQ[").replace("], F[1], ", "], nrpF1, ") for ln in acc_lines]
        acc_lines.insert(0, "    const R nrpF1 = -rp * F[1];")
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


def shell_range(lo, hi):
    """Cartesian triples of every total angular momentum in [lo, hi] (empty if hi < lo or lo < 0)."""
    if lo < 0 or hi < lo:
        return []
    return [c for l in range(lo, hi + 1) for c in comps(l)]


def gen_hrr_from(E, la, lb, lc, ld, src, eidx, fidx, nf, tag):
    """HRR of class (la lb|lc ld) reading [e0|f0] from ``src[eidx[e]*nf + fidx[f]]``.

    Returns {(a, b, c, d): expression name} for every component; temporaries are
    prefixed with ``tag`` so several instances can share one function body."""
    bra_memo = {}

    def bra(a, b, f):
        key = (a, b, f)
        if key in bra_memo:
            return bra_memo[key]
        if sum(b) == 0:
            r = "%s[%d]" % (src, eidx[a] * nf + fidx[f])
            bra_memo[key] = r
            return r
        i = pick_axis(b)
        b1 = add(b, i, -1)
        x = bra(add(a, i, 1), b1, f)
        y = bra(a, b1, f)
        name = "%sh%s%s_%s" % (tag, nm(a), nm(b), nm(f))
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
        name = "%sk%s%s%s%s" % (tag, nm(a), nm(b), nm(c), nm(d))
        E.lines.append("    const R %s = %s + CD[%d] * %s;" % (name, x, i, y))
        E.flops += 2
        ket_memo[key] = name
        return name

    out = {}
    for a in comps(la):
        for b in comps(lb):
            for c in comps(lc):
                for d in comps(ld):
                    out[(a, b, c, d)] = ket(a, b, c, d)
    return out


def gen_grad(la, lb, lc, ld):
    """Derivative integrals of class (la lb|lc ld) w.r.t. centres A, B, C,
    contracted with the two-particle density.

    With d/dA_i phi_a = 2 alpha phi_{a+1_i} - a_i phi_{a-1_i}, the primitive
    integrals are accumulated with weights 2alpha (A raised), 2beta (B raised),
    2gamma (C raised) and 1 (lowered terms); HRR then yields
      (a+1_i b|cd), (a b+1_i|cd), (ab|c+1_i d) and the lowered classes, and
      g_A[i] = sum_abcd Gam_abcd [(a+1_i b|cd) - a_i (a-1_i b|cd)]   (B, C alike).
    The D centre follows from translational invariance in the kernel."""
    V = Emitter()
    memo = {}
    consts = set()

    def const(kind, k):
        name = "%s_%d" % (kind, k)
        if name not in consts:
            consts.add(name)
            V.lines.append("    const R %s = R(%d) * %s;" % (name, k, kind))
            V.flops += 1
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
        if sum(f) > 0:
            i = pick_axis(f)
            f1 = add(f, i, -1)
            expr = "QC[%d] * %s + WQ[%d] * %s" % (i, get(e, f1, m), i, get(e, f1, m + 1))
            fl = 3
            if f1[i] > 0:
                f2 = add(f1, i, -1)
                expr += " + %s * (%s - rq * %s)" % (const("o2q", f1[i]), get(e, f2, m), get(e, f2, m + 1))
                fl += 4
            if e[i] > 0:
                expr += " + %s * %s" % (const("o2pq", e[i]), get(add(e, i, -1), f1, m + 1))
                fl += 2
        else:
            i = pick_axis(e)
            e1 = add(e, i, -1)
            expr = "PA[%d] * %s + WP[%d] * %s" % (i, get(e1, f, m), i, get(e1, f, m + 1))
            fl = 3
            if e1[i] > 0:
                e2 = add(e1, i, -1)
                expr += " + %s * (%s - rp * %s)" % (const("o2p", e1[i]), get(e2, f, m), get(e2, f, m + 1))
                fl += 4
        V.lines.append("    const R %s = %s;" % (name, expr))
        V.flops += fl
        memo[key] = name
        return name

    # accumulator sets: (name, weight, e-range, f-range)
    sets = {
        "accA": ("wa", shell_range(la + 1, la + lb + 1), shell_range(lc, lc + ld)),
        "accB": ("wb", shell_range(la, la + lb + 1), shell_range(lc, lc + ld)),
        "accC": ("wc", shell_range(la, la + lb), shell_range(lc + 1, lc + ld + 1)),
    }
    # the unweighted set covers the three lowered classes
    e0 = set(shell_range(la - 1, la - 1 + lb)) | set(shell_range(la, la + lb - 1) if lb > 0 else []) | \
        set(shell_range(la, la + lb) if lc > 0 else [])
    f0 = set(shell_range(lc, lc + ld)) | set(shell_range(lc - 1, lc - 1 + ld) if lc > 0 else [])
    e0 = sorted(e0, key=lambda c: (sum(c), comps(sum(c)).index(c)))
    f0 = sorted(f0, key=lambda c: (sum(c), comps(sum(c)).index(c)))
    sets["acc0"] = (None, e0, f0)
    sizes = {}
    maps = {}
    for name, (w, es, fs) in sets.items():
        maps[name] = ({c: i for i, c in enumerate(es)}, {c: i for i, c in enumerate(fs)}, len(fs))
        sizes[name] = len(es) * len(fs)
    acc_lines = []
    needed0 = set()
    if la > 0:
        needed0 |= {(e, f) for e in shell_range(la - 1, la - 1 + lb) for f in shell_range(lc, lc + ld)}
    if lb > 0:
        needed0 |= {(e, f) for e in shell_range(la, la + lb - 1) for f in shell_range(lc, lc + ld)}
    if lc > 0:
        needed0 |= {(e, f) for e in shell_range(la, la + lb) for f in shell_range(lc - 1, lc - 1 + ld)}
    for name, (w, es, fs) in sets.items():
        em, fm, nf = maps[name]
        for e in es:
            for f in fs:
                if name == "acc0" and (e, f) not in needed0:
                    continue
                v = get(e, f, 0)
                if w is None:
                    acc_lines.append("    %s[%d] += %s;" % (name, em[e] * nf + fm[f], v))
                    V.flops += 1
                else:
                    acc_lines.append("    %s[%d] = fma(%s, %s, %s[%d]);" % (name, em[e] * nf + fm[f], w, v, name,
                                                                         em[e] * nf + fm[f]))
                    V.flops += 2
    V.lines.extend(acc_lines)

    H = Emitter()
    NA, NB, NC, ND = ncart(la), ncart(lb), ncart(lc), ncart(ld)
    em, fm, nf = maps["accA"]
    Ap = gen_hrr_from(H, la + 1, lb, lc, ld, "accA", em, fm, nf, "ap")
    em, fm, nf = maps["accB"]
    Bp = gen_hrr_from(H, la, lb + 1, lc, ld, "accB", em, fm, nf, "bp")
    em, fm, nf = maps["accC"]
    Cp = gen_hrr_from(H, la, lb, lc + 1, ld, "accC", em, fm, nf, "cp")
    em, fm, nf = maps["acc0"]
    Am = gen_hrr_from(H, la - 1, lb, lc, ld, "acc0", em, fm, nf, "am") if la > 0 else {}
    Bm = gen_hrr_from(H, la, lb - 1, lc, ld, "acc0", em, fm, nf, "bm") if lb > 0 else {}
    Cm = gen_hrr_from(H, la, lb, lc - 1, ld, "acc0", em, fm, nf, "cm") if lc > 0 else {}
    for ia, a in enumerate(comps(la)):
        for ib, b in enumerate(comps(lb)):
            for ic, c in enumerate(comps(lc)):
                for id_, d in enumerate(comps(ld)):
                    k = ((ia * NB + ib) * NC + ic) * ND + id_
                    for i in range(3):
                        t = Ap[(add(a, i, 1), b, c, d)]
                        if a[i] > 0:
                            t = "(%s - R(%d) * %s)" % (t, a[i], Am[(add(a, i, -1), b, c, d)])
                            H.flops += 2
                        H.lines.append("    g[%d] = fma(gam[%d], %s, g[%d]);" % (i, k, t, i))
                        t = Bp[(a, add(b, i, 1), c, d)]
                        if b[i] > 0:
                            t = "(%s - R(%d) * %s)" % (t, b[i], Bm[(a, add(b, i, -1), c, d)])
                            H.flops += 2
                        H.lines.append("    g[%d] = fma(gam[%d], %s, g[%d]);" % (3 + i, k, t, 3 + i))
                        t = Cp[(a, b, add(c, i, 1), d)]
                        if c[i] > 0:
                            t = "(%s - R(%d) * %s)" % (t, c[i], Cm[(a, b, add(c, i, -1), d)])
                            H.flops += 2
                        H.lines.append("    g[%d] = fma(gam[%d], %s, g[%d]);" % (6 + i, k, t, 6 + i))
                        H.flops += 6
    return V, H, sizes, la + lb + lc + ld + 1


def pair_classes(lmax):
    return [(a, b) for a in range(lmax + 1) for b in range(a + 1)]


def quartet_classes(lmax):
    pcs = pair_classes(lmax)
    out = []
    for i, x in enumerate(pcs):
        for y in pcs[: i + 1]:
            out.append(x + y)
    return out


GRAD_LMAX = 1  # gradient recurrences are generated for classes with every l <= GRAD_LMAX
AD_LMAX = 7  # classes above take the finite-difference gradient kernel (compile time of the dual-number form)
SPLIT_L = 5  # classes with la+lb+lc+ld >= SPLIT_L compile in four units each


def main(outdir, lmax):
    os.makedirs(outdir, exist_ok=True)
    for f in os.listdir(outdir):
        if f.startswith(("inst_", "cls_")) or f == "eri_classes.cuh":
            os.remove(os.path.join(outdir, f))
    classes = quartet_classes(lmax)
    model = {}
    for (la, lb, lc, ld) in classes:
        V, ne, nf, L = gen_vrr(la, lb, lc, ld)
        H = gen_hrr(la, lb, lc, ld)
        name = "Cls_%d_%d_%d_%d" % (la, lb, lc, ld)
        hdr = ["// Generated by gen_eri.py: Obara-Saika VRR + HGP HRR of class (%d%d|%d%d). Do not edit." % (la, lb, lc, ld),
               "#pragma once", ""]
        hdr.append("struct %s {" % name)
        hdr.append("  static constexpr int LA = %d, LB = %d, LC = %d, LD = %d, L = %d;" % (la, lb, lc, ld, L))
        hdr.append("  static constexpr int NE = %d, NF = %d;" % (ne, nf))
        hdr.append("  static constexpr int NA = %d, NB = %d, NC = %d, ND = %d;" % (ncart(la), ncart(lb), ncart(lc), ncart(ld)))
        hdr.append("  template <typename R>")
        hdr.append("  __device__ __forceinline__ static void vrr(const R* __restrict__ F, const R* PA, const R* WP, const R* QC, const R* WQ,")
        hdr.append("                                             const R* PQ, R o2p, R o2q, R o2pq, R rp, R rq, R* acc) {")
        hdr.append("    (void)PA; (void)WP; (void)QC; (void)WQ; (void)PQ; (void)o2p; (void)o2q; (void)o2pq; (void)rp; (void)rq;")
        hdr.extend(V.lines)
        hdr.append("  }")
        hdr.append("  template <typename R>")
        hdr.append("  __device__ __forceinline__ static void hrr(const R* __restrict__ acc, const R* AB, const R* CD, R* out) {")
        hdr.append("    (void)AB; (void)CD;")
        hdr.extend(H.lines)
        hdr.append("  }")
        entry = {"L": L, "vrr_flops_per_prim_quartet": V.flops, "hrr_flops_per_quartet": H.flops,
                 "n_eri_per_quartet": ncart(la) * ncart(lb) * ncart(lc) * ncart(ld)}
        has_grad = max(la, lb, lc, ld) <= GRAD_LMAX
        hdr.append("  static constexpr bool HAS_GRAD = %s;" % ("true" if has_grad else "false"))
        if has_grad:
            GV, GH, gsizes, LG = gen_grad(la, lb, lc, ld)
            hdr.append("  // nuclear-gradient recurrences (derivatives w.r.t. centres A, B, C)")
            hdr.append("  static constexpr int LG = %d;" % LG)
            hdr.append("  static constexpr int NACC0 = %d, NACCA = %d, NACCB = %d, NACCC = %d;" % (
                max(1, gsizes["acc0"]), gsizes["accA"], gsizes["accB"], gsizes["accC"]))
            hdr.append("  template <typename R>")
            hdr.append("  __device__ __forceinline__ static void vrr_grad(const R* __restrict__ F, const R* PA, const R* WP, const R* QC,")
            hdr.append("      const R* WQ, R o2p, R o2q, R o2pq, R rp, R rq, R wa, R wb, R wc, R* acc0, R* accA, R* accB, R* accC) {")
            hdr.append("    (void)PA; (void)WP; (void)QC; (void)WQ; (void)o2p; (void)o2q; (void)o2pq; (void)rp; (void)rq; (void)acc0;")
            hdr.extend(GV.lines)
            hdr.append("  }")
            hdr.append("  template <typename R>")
            hdr.append("  __device__ __forceinline__ static void hrr_grad(const R* __restrict__ acc0, const R* __restrict__ accA,")
            hdr.append("      const R* __restrict__ accB, const R* __restrict__ accC, const R* AB, const R* CD, const R* gam, R* g) {")
            hdr.append("    (void)AB; (void)CD; (void)acc0;")
            hdr.extend(GH.lines)
            hdr.append("  }")
            entry.update({"grad_vrr_flops_per_prim_quartet": GV.flops, "grad_hrr_flops_per_quartet": GH.flops})
        else:
            hdr.append("  static constexpr int LG = L + 1, NACC0 = 1, NACCA = 1, NACCB = 1, NACCC = 1;")
            hdr.append("  template <typename R>")
            hdr.append("  __device__ __forceinline__ static void vrr_grad(const R*, const R*, const R*, const R*, const R*, R, R, R, R, R,")
            hdr.append("                                                  R, R, R, R*, R*, R*, R*) {}")
            hdr.append("  template <typename R>")
            hdr.append("  __device__ __forceinline__ static void hrr_grad(const R*, const R*, const R*, const R*, const R*, const R*,")
            hdr.append("                                                  const R*, R*) {}")
        hdr.append("};")
        model["(%d%d|%d%d)" % (la, lb, lc, ld)] = entry
        with open(os.path.join(outdir, "cls_%d%d%d%d.cuh" % (la, lb, lc, ld)), "w") as f:
            f.write("\n".join(hdr) + "\n")
    # one instantiation unit per class so nvcc can compile them in parallel
    names = []
    for (la, lb, lc, ld) in classes:
        name = "Cls_%d_%d_%d_%d" % (la, lb, lc, ld)
        names.append(name)
        # the large classes compile their four launch pieces in units of their own
        split = la + lb + lc + ld >= SPLIT_L
        sig = "(const ClassLaunch&, const EriArgs&, int, int, cudaStream_t)"
        with open(os.path.join(outdir, "inst_%d%d%d%d.cu" % (la, lb, lc, ld)), "w") as f:
            f.write('// Generated by gen_eri.py. Do not edit.\n#include "cls_%d%d%d%d.cuh"\n#include "../eri_kernel.cuh"\n'
                    % (la, lb, lc, ld))
            f.write("namespace fockgb {\n")
            if split:
                for part in range(4):
                    f.write("extern template cudaError_t launch_part<%s, %d>%s;\n" % (name, part, sig))
            f.write("cudaError_t launch_%s(const ClassLaunch& cl, const EriArgs& a, int mode, int prec, cudaStream_t s) {\n" % name)
            f.write("  return launch_class<%s>(cl, a, mode, prec, s);\n}\n" % name)
            f.write("}  // namespace fockgb\n")
        if split:
            for part in range(4):
                with open(os.path.join(outdir, "inst_%d%d%d%d_p%d.cu" % (la, lb, lc, ld, part)), "w") as f:
                    f.write('// Generated by gen_eri.py. Do not edit.\n#include "cls_%d%d%d%d.cuh"\n'
                            '#include "../eri_kernel.cuh"\n' % (la, lb, lc, ld))
                    f.write("namespace fockgb {\ntemplate cudaError_t launch_part<%s, %d>%s;\n}  // namespace fockgb\n"
                            % (name, part, sig))
        if max(la, lb, lc, ld) > GRAD_LMAX and la + lb + lc + ld <= AD_LMAX:
            # gradient kernel of the class by dual-number differentiation of its
            # recurrences (eri_grad_ad.cuh), in a unit of its own
            with open(os.path.join(outdir, "inst_ad_%d%d%d%d.cu" % (la, lb, lc, ld)), "w") as f:
                f.write('// Generated by gen_eri.py. Do not edit.\n#include "cls_%d%d%d%d.cuh"\n'
                        '#include "../eri_grad_ad.cuh"\n' % (la, lb, lc, ld))
                f.write("namespace fockgb {\n")
                f.write("template cudaError_t launch_grad_ad<%s>(const ClassLaunch&, const EriArgs&, cudaStream_t);\n"
                        % name)
                f.write("}  // namespace fockgb\n")
        elif max(la, lb, lc, ld) > GRAD_LMAX:
            # (dd|dd): the dual-number form compiles for 5-8 minutes; the
            # fourth-order finite difference of the class's integrals instead
            with open(os.path.join(outdir, "inst_fd_%d%d%d%d.cu" % (la, lb, lc, ld)), "w") as f:
                f.write('// Generated by gen_eri.py. Do not edit.\n#include "cls_%d%d%d%d.cuh"\n'
                        '#include "../eri_grad_fd.cuh"\n' % (la, lb, lc, ld))
                f.write("namespace fockgb {\n")
                f.write("template cudaError_t launch_grad_fd<%s>(const ClassLaunch&, const EriArgs&, cudaStream_t);\n"
                        % name)
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
        f.write("constexpr int kGeneratedGradLmax = %d;\n" % GRAD_LMAX)
        f.write("constexpr int kGradAdLmax = %d;\n" % AD_LMAX)
        f.write("}  // namespace fockgb\n")
    with open(os.path.join(outdir, "roofline_model.json"), "w") as f:
        json.dump(model, f, indent=1, sort_keys=True)
    return classes


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 2)
