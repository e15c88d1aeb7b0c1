"""Generates sgh_hex_geometry.cuh: straight-line device code for one hex's
outward corner area normals B (geometry.cpp:40-234), exact volume
(geometry.cpp:271-310) and the velocity-divergence sums (momentum.cpp:221-292).

Every expression keeps the reference's operands and association order, so the
generated code is bit-for-bit equivalent to it when compiled without
contraction.  The work is shared where that is exact:
  * each cofactor combo is evaluated once per unordered node pair; the other
    orientation is its exact negation (term-by-term negated sums round to the
    negated value);
  * the volume reuses the B-matrix products y_j * comb_ij of component 0.
The volume's products and sums (and with them component 0 of B) go through
FX_MUL / FX_ADD, which stay separately rounded in the fused-multiply-add build
too: the cofactor sum cancels terms of size ~|x| h^2 down to a volume ~h^3, so
contracting it would move the volume (and the density) by ~|x|/h ulps, 1e-11
relative on a 256^3 mesh, while every other field moves by ~1e-16.

The tables are parsed from sgh_hex.h so there is one source of truth.
Run:  python gen_hex_geometry.py   (writes sgh_hex_geometry.cuh beside it)
"""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_tables():
    src = open(os.path.join(HERE, "sgh_hex.h")).read()

    def arr(name):
        m = re.search(r"constexpr[^=]*\b%s\b[^=]*=\s*\{(.*?)\};" % name, src, re.S)
        return [int(v) for v in re.findall(r"-?\d+", m.group(1))]

    J = arr("J")
    T = arr("TERMS")
    VI = arr("VI")
    VJ = arr("VJ")
    J = [J[p * 6:(p + 1) * 6] for p in range(8)]
    T = [[T[(p * 6 + t) * 4:(p * 6 + t + 1) * 4] for t in range(6)] for p in range(8)]
    VJ = [VJ[a * 6:(a + 1) * 6] for a in range(8)]
    return J, T, VI, VJ


def main():
    J, T, VI, VJ = parse_tables()
    # unordered pairs, stored in the p < j orientation
    pairs = []  # (p, t, j)
    pair_of = {}
    for p in range(8):
        for t in range(6):
            j = J[p][t]
            if p < j:
                pair_of[(p, j)] = len(pairs)
                pairs.append((p, t, j))
    for p in range(8):
        for t in range(6):
            j = J[p][t]
            if p > j:
                k = pair_of[(j, p)]
                a = T[j][pairs[k][1]]
                b = T[p][t]
                assert [-v for v in a if v] == [v for v in b if v], (p, j)
    comps = [("y", "z"), ("z", "x"), ("x", "y")]  # (O, I) for c = 0, 1, 2
    L = []
    w = L.append
    w("// GENERATED by gen_hex_geometry.py from sgh_hex.h -- do not edit.")
    w("// Straight-line hex geometry; see the generator's docstring for the exactness argument.")
    w("#pragma once")
    w("")
    w("// Separately rounded product and sum, also where the unit contracts (FIERRO_FMA=1).")
    w("#if FIERRO_FMA")
    w("#define FX_MUL(a, b) __dmul_rn((a), (b))")
    w("#define FX_ADD(a, b) __dadd_rn((a), (b))")
    w("#else")
    w("#define FX_MUL(a, b) ((a) * (b))")
    w("#define FX_ADD(a, b) ((a) + (b))")
    w("#endif")
    w("")
    w("// In: x,y,z,u,v,w[8] (node lids 0..7).  Out: vol; bmat rows lid*3+dim at")
    w("// bmat[row*ne + e]; Sx,Sy,Sz = sum_p u_p B(p,0), v_p B(p,1), w_p B(p,2) (p order).")
    w("__device__ __forceinline__ void hex_geometry(const double* __restrict__ x, const double* __restrict__ y,")
    w("    const double* __restrict__ z, const double* __restrict__ u, const double* __restrict__ v,")
    w("    const double* __restrict__ w, double* __restrict__ bmat, int ne, int e, double& vol,")
    w("    double& Sx, double& Sy, double& Sz) {")
    w("  const double twelth = 1. / 12.;")
    vel = {0: "u", 1: "v", 2: "w"}
    for c, (O, I) in enumerate(comps):
        w("  {  // component %d: O = %s, I = %s" % (c, O, I))
        for k, (p, t, j) in enumerate(pairs):
            terms = [v for v in T[p][t] if v]
            expr = ("-" if terms[0] < 0 else "") + "%s[%d]" % (I, abs(terms[0]) - 1)
            for v_ in terms[1:]:
                expr = "(%s %s %s[%d])" % (expr, "+" if v_ > 0 else "-", I, abs(v_) - 1)
            w("    const double cm%d = %s;  // pair (%d,%d)" % (k, expr, p, j))
        # products
        for p in range(8):
            for t in range(6):
                j = J[p][t]
                if p < j:
                    cm = "cm%d" % pair_of[(p, j)]
                else:
                    cm = "(-cm%d)" % pair_of[(j, p)]
                if c == 0:
                    w("    const double pr%d_%d = FX_MUL(%s[%d], %s);" % (p, t, O, j, cm))
                else:
                    w("    const double pr%d_%d = %s[%d] * %s;" % (p, t, O, j, cm))
        if c == 0:
            # volume: sum_a x[VI[a]] * (sum_b products in VJ order)
            for a in range(8):
                i = VI[a]
                slots = [J[i].index(jj) for jj in VJ[a]]
                expr = "pr%d_%d" % (i, slots[0])
                for s_ in slots[1:]:
                    expr = "FX_ADD(%s, pr%d_%d)" % (expr, i, s_)
                w("    const double vi%d = FX_MUL(x[%d], %s);" % (a, i, expr))
            expr = "vi0"
            for a in range(1, 8):
                expr = "FX_ADD(%s, vi%d)" % (expr, a)
            w("    vol = FX_MUL(%s, twelth);" % expr)
        S = "S" + "xyz"[c]
        for p in range(8):
            expr = "pr%d_0" % p
            for t in range(1, 6):
                expr = "(%s + pr%d_%d)" % (expr, p, t)
            w("    const double b%d = %s * twelth;" % (p, expr))
            w("    bmat[(size_t)%d * ne + e] = b%d;" % (p * 3 + c, p))
            if p == 0:
                w("    %s = %s[0] * b0;" % (S, vel[c]))
            else:
                w("    %s = %s + %s[%d] * b%d;" % (S, S, vel[c], p, p))
        w("  }")
    w("}")
    w("")
    w("// The exact hex volume alone (geometry.cpp:271-310), the same operations in the")
    w("// same order as hex_geometry's volume.")
    w("__device__ __forceinline__ double hex_volume(const double* __restrict__ x, const double* __restrict__ y,")
    w("    const double* __restrict__ z) {")
    w("  const double twelth = 1. / 12.;")
    O, I = comps[0]
    for k, (p_, t, j) in enumerate(pairs):
        terms = [v for v in T[p_][t] if v]
        expr = ("-" if terms[0] < 0 else "") + "%s[%d]" % (I, abs(terms[0]) - 1)
        for v_ in terms[1:]:
            expr = "(%s %s %s[%d])" % (expr, "+" if v_ > 0 else "-", I, abs(v_) - 1)
        w("  const double cm%d = %s;" % (k, expr))
    used = set()
    for a in range(8):
        i = VI[a]
        for jj in VJ[a]:
            used.add((i, J[i].index(jj)))
    for (p_, t) in sorted(used):
        j = J[p_][t]
        cm = ("cm%d" % pair_of[(p_, j)]) if p_ < j else ("(-cm%d)" % pair_of[(j, p_)])
        w("  const double pr%d_%d = %s[%d] * %s;" % (p_, t, O, j, cm))
    for a in range(8):
        i = VI[a]
        slots = [J[i].index(jj) for jj in VJ[a]]
        expr = "pr%d_%d" % (i, slots[0])
        for s_ in slots[1:]:
            expr = "(%s + pr%d_%d)" % (expr, i, s_)
        w("  const double vi%d = x[%d] * %s;" % (a, i, expr))
    expr = "vi0"
    for a in range(1, 8):
        expr = "(%s + vi%d)" % (expr, a)
    w("  return %s * twelth;" % expr)
    w("}")
    w("")
    w("// Reverse mode of the corner normals: given Bbar[lid*3+dim] (the adjoint of")
    w("// B(lid, dim)), accumulate the coordinate adjoints xbar, ybar, zbar[8].  B is")
    w("// bilinear, B(p,c) = sum_t O[j_t] comb_t(I) / 12, and each unordered pair (p, j)")
    w("// enters B(p) as O[j] cm and B(j) as -O[p] cm with one shared combo cm, so")
    w("//   Obar[j] += g_p cm,  Obar[p] -= g_j cm,  Ibar[terms of cm] +-= g_p O[j] - g_j O[p]")
    w("// with g = Bbar / 12 (multiply-adds fused: the adjoint has no parity target).")
    w("__device__ __forceinline__ void hex_bmatrix_adjoint(const double* __restrict__ x, const double* __restrict__ y,")
    w("    const double* __restrict__ z, const double* __restrict__ Bbar, double* __restrict__ xbar,")
    w("    double* __restrict__ ybar, double* __restrict__ zbar) {")
    w("  const double twelth = 1. / 12.;")
    bar = {"x": "xbar", "y": "ybar", "z": "zbar"}
    for c, (O, I) in enumerate(comps):
        w("  {  // component %d: O = %s, I = %s" % (c, O, I))
        for p_ in range(8):
            w("    const double g%d = Bbar[%d] * twelth;" % (p_, p_ * 3 + c))
        for k, (p_, t, j) in enumerate(pairs):
            terms = [v for v in T[p_][t] if v]
            expr = ("-" if terms[0] < 0 else "") + "%s[%d]" % (I, abs(terms[0]) - 1)
            for v_ in terms[1:]:
                expr = "(%s %s %s[%d])" % (expr, "+" if v_ > 0 else "-", I, abs(v_) - 1)
            w("    {  // pair (%d,%d)" % (p_, j))
            w("      const double cm = %s;" % expr)
            w("      %s[%d] = fma(g%d, cm, %s[%d]);" % (bar[O], j, p_, bar[O], j))
            w("      %s[%d] = fma(-g%d, cm, %s[%d]);" % (bar[O], p_, j, bar[O], p_))
            w("      const double wk = fma(g%d, %s[%d], -(g%d * %s[%d]));" % (p_, O, j, j, O, p_))
            for v_ in terms:
                w("      %s[%d] %s= wk;" % (bar[I], abs(v_) - 1, "+" if v_ > 0 else "-"))
            w("    }")
        w("  }")
    w("}")
    out = os.path.join(HERE, "sgh_hex_geometry.cuh")
    with open(out, "w") as f:
        f.write("\n".join(L) + "\n")
    print("wrote", out, "pairs", len(pairs))


if __name__ == "__main__":
    main()
