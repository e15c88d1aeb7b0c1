"""Generates sgh_hex_geometry.cuh: straight-line device code for one hex's
outward corner area normals B (geometry.cpp:40-234), exact volume
(geometry.cpp:271-310), velocity divergence (momentum.cpp:221-292) and the
squared node-pair distances of the CFL time step (time_integration.cpp:93-128).

Every expression keeps the reference's operands and association order, so the
generated code is bit-for-bit equivalent to it when compiled without
contraction.  The work is shared where that is exact:
  * each cofactor combo is evaluated once per unordered node pair; the other
    orientation is its exact negation (term-by-term negated sums round to the
    negated value);
  * the volume reuses the B-matrix products y_j * comb_ij of component 0;
  * the 12 two-term combos are face-diagonal coordinate differences, reused (up
    to sign, which squaring removes) by the CFL distances.

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
    PA = arr("PAIR_A")
    PB = arr("PAIR_B")
    J = [J[p * 6:(p + 1) * 6] for p in range(8)]
    T = [[T[(p * 6 + t) * 4:(p * 6 + t + 1) * 4] for t in range(6)] for p in range(8)]
    VJ = [VJ[a * 6:(a + 1) * 6] for a in range(8)]
    return J, T, VI, VJ, PA, PB


def main():
    J, T, VI, VJ, PA, PB = parse_tables()
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
    w("// In: x,y,z,u,v,w[8] (node lids 0..7).  Out: vol; bmat rows lid*3+dim at")
    w("// bmat[row*ne + e]; Sx,Sy,Sz = sum_p u_p B(p,0), v_p B(p,1), w_p B(p,2) (p order);")
    w("// with CFL, d2min = min over the 28 node pairs of the squared distance.")
    w("template <bool CFL>")
    w("__device__ __forceinline__ void hex_geometry(const double* __restrict__ x, const double* __restrict__ y,")
    w("    const double* __restrict__ z, const double* __restrict__ u, const double* __restrict__ v,")
    w("    const double* __restrict__ w, double* __restrict__ bmat, int ne, int e, double& vol,")
    w("    double& Sx, double& Sy, double& Sz, double& d2min) {")
    w("  const double twelth = 1. / 12.;")
    # two-term combos hold face-diagonal differences: map node pair -> (component, var)
    diag = {}
    vel = {0: "u", 1: "v", 2: "w"}
    for c, (O, I) in enumerate(comps):
        w("  {  // component %d: O = %s, I = %s" % (c, O, I))
        for k, (p, t, j) in enumerate(pairs):
            terms = [v for v in T[p][t] if v]
            expr = ("-" if terms[0] < 0 else "") + "%s[%d]" % (I, abs(terms[0]) - 1)
            for v_ in terms[1:]:
                expr = "(%s %s %s[%d])" % (expr, "+" if v_ > 0 else "-", I, abs(v_) - 1)
            w("    const double cm%d = %s;  // pair (%d,%d)" % (k, expr, p, j))
            if len(terms) == 2:
                a, b = abs(terms[0]) - 1, abs(terms[1]) - 1
                diag[(min(a, b), max(a, b), I)] = "cm%d" % k
        # products
        for p in range(8):
            for t in range(6):
                j = J[p][t]
                if p < j:
                    cm = "cm%d" % pair_of[(p, j)]
                else:
                    cm = "(-cm%d)" % pair_of[(j, p)]
                w("    const double pr%d_%d = %s[%d] * %s;" % (p, t, O, j, cm))
        if c == 0:
            # volume: sum_a x[VI[a]] * (sum_b products in VJ order)
            for a in range(8):
                i = VI[a]
                slots = [J[i].index(jj) for jj in VJ[a]]
                expr = "pr%d_%d" % (i, slots[0])
                for s in slots[1:]:
                    expr = "(%s + pr%d_%d)" % (expr, i, s)
                w("    const double vi%d = x[%d] * %s;" % (a, i, expr))
            expr = "vi0"
            for a in range(1, 8):
                expr = "(%s + vi%d)" % (expr, a)
            w("    vol = %s * twelth;" % expr)
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
        if c < 2:
            # keep the face-diagonal differences of this component for the CFL pass
            pass
        names = []
        for (a, b, I_), var in sorted(diag.items()):
            if I_ == I:
                names.append((a, b, var))
        for a, b, var in names:
            w("    const double fd_%s_%d_%d = %s;" % (I, a, b, var))
        w("    (void)0;")
        # hoist the face-diagonal differences out of the block scope
        L[-1] = "    " + " ".join("d%s_%d_%d = fd_%s_%d_%d;" % (I, a, b, I, a, b) for a, b, _ in names)
        w("  }")
    # declare hoisted vars at the top: insert after the opening line
    decl = []
    for I in ("z", "x", "y"):
        for (a, b, I_), _ in sorted(diag.items()):
            if I_ == I:
                decl.append("d%s_%d_%d" % (I, a, b))
    insert_at = L.index("  const double twelth = 1. / 12.;") + 1
    L.insert(insert_at, "  double " + ", ".join(decl) + ";")
    # CFL
    w("  if (CFL) {")
    w("    // squared distances (dx*dx + dy*dy) + dz*dz of time_integration.cpp:107-109,")
    w("    // pow(d, 2.0) == d*d; minimum taken on the order keys of the non-negative values")
    w("    long long kmin = 0x7FFFFFFFFFFFFFFFLL;")
    for i in range(28):
        a, b = PA[i], PB[i]
        comps_expr = []
        for I in ("x", "y", "z"):
            key = (min(a, b), max(a, b), I)
            if key in diag:
                comps_expr.append("d%s_%d_%d" % (I, min(a, b), max(a, b)))
            else:
                comps_expr.append("(%s[%d] - %s[%d])" % (I, b, I, a))
        w("    { const double dx = %s, dy = %s, dz = %s;" % tuple(comps_expr))
        w("      const double d2 = (dx * dx + dy * dy) + dz * dz;")
        w("      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (%d,%d)" % (a, b))
    w("    d2min = okey_decode(kmin);")
    w("  } else {")
    w("    d2min = 0.0;")
    # silence unused warnings
    w("    (void)(" + " + ".join(decl) + ");")
    w("  }")
    w("}")
    out = os.path.join(HERE, "sgh_hex_geometry.cuh")
    with open(out, "w") as f:
        f.write("\n".join(L) + "\n")
    print("wrote", out, "pairs", len(pairs), "face diagonals", len(diag))


if __name__ == "__main__":
    main()
