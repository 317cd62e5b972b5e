"""Derives the per-star part of the force VJP and writes pn_finish_vjp_gen.cuh.

The finishing kernel (pn_kernels.cu, finish_body) turns, for star i, the pair sums
(G, Phi, S0, U, W), the star's own state (s = x_i - x_0, v, m_i), the BH mass m0 and the
global sums (A1, C, B3, P) into
    a_i  = G - m0 R^3 s + inv_c2 * pn_i            (the star's acceleration)
    bh_i                                            (its share of the BH's 1PN acceleration)
with R = (|s|^2 + eps^2)^(-1/2) -- the closed forms of Limit-sticky9.c:213-422 (stars) and
:54-207 (BH) after the pair sums.  For adjoints abar_i (of a_i) and abar_0 (of the BH's
acceleration a_0 = B3 + inv_c2 * sum_i bh_i) this script differentiates
    L_i = abar_i . a_i + inv_c2 * abar_0 . bh_i
with respect to every input and prints C with common subexpressions eliminated.  The formulas
below are the same expressions as finish_body; tests/test_adjoint_gpu.py checks the result
against central finite differences of the force.

    python pn_gb300/csrc/gen_finish_vjp.py     (needs sympy; the output is committed)
"""
import os

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "pn_finish_vjp_gen.cuh")


def vec(name):
    return sp.Matrix(sp.symbols(f"{name}0:3", real=True))


def forward():
    s, v, G, W, B3, P = (vec(n) for n in ("s", "v", "G", "W", "gB", "gP"))
    Phi, S0, U, mi, m0, eps, eps2, ic2, A1, C = sp.symbols(
        "Phi S0 U mi m0 eps eps2 ic2 gA gC", real=True)
    q = s.dot(s)
    R = 1 / sp.sqrt(q + eps2)
    R3 = R ** 3
    vi2 = v.dot(v)
    vis = v.dot(s)
    viP = v.dot(P)
    Ps = P.dot(s)
    sB3 = s.dot(B3)
    sG = s.dot(G)
    h = sp.Rational(1, 2)
    cs = (-m0 * R3 * (4 * m0 * R - vi2) + 5 * m0 * R3 * mi * R - 4 * mi * R3 * vi2
          - m0 * R3 * (4 * Phi + sp.Rational(5, 4) * A1 - sp.Rational(1, 4) * C + h * sB3)
          + sp.Rational(7, 2) * m0 * U + 4 * R3 * viP
          + mi * R3 * m0 * (4 / eps + sp.Rational(5, 4) * R + sp.Rational(1, 4) * q * R3)
          - sp.Rational(7, 2) * mi * R3 * m0 * (1 / eps - R) - 4 * mi * R3 * vi2)
    cv = -4 * m0 * R3 * vis + 7 * mi * R3 * vis - 3 * R3 * Ps + 7 * mi * R3 * vis
    pn = cs * s + cv * v + 4 * m0 * R * G - sp.Rational(7, 2) * m0 * R * B3 - 4 * R3 * vis * P + W
    a = G - m0 * R3 * s + ic2 * pn
    T = -2 * sG - (Phi - eps2 * S0)
    mR3 = mi * R3
    bs = (mR3 * (5 * m0 * R - 2 * vi2 + sp.Rational(3, 2) * vis * vis / q) + 4 * mR3 * R * mi
          + mR3 * (4 * A1 + sp.Rational(5, 4) * Phi + sp.Rational(1, 4) * T) - (mR3 / m0) * 4 * viP
          + mR3 * mi * (4 * R + sp.Rational(5, 4) * eps) - (mR3 * mi / m0) * 4 * vi2)
    bv = 3 * mR3 * vis + (mR3 / m0) * 4 * Ps + (mR3 * mi / m0) * 7 * vis
    bh = bs * s + bv * v - sp.Rational(7, 2) * R * mi * G + (mR3 / m0) * 3 * vis * P
    ins = dict(s=s, v=v, G=G, W=W, gB=B3, gP=P, Phi=Phi, S0=S0, U=U, m0=m0, gA=A1, gC=C)
    return a, bh, ins, ic2


def main():
    a, bh, ins, ic2 = forward()
    ab, bb = vec("ab"), vec("bb")
    L = ab.dot(a) + ic2 * bb.dot(bh)
    outs, names = [], []
    for nm in ("s", "v", "G", "W", "gB", "gP"):
        for k in range(3):
            outs.append(sp.diff(L, ins[nm][k]))
            names.append(f"{nm}_b[{k}]")
    for nm in ("Phi", "S0", "U", "m0", "gA", "gC"):
        outs.append(sp.diff(L, ins[nm]))
        names.append(f"{nm}_b")
    repl, red = sp.cse(outs, symbols=sp.numbered_symbols("t"), optimizations="basic")
    lines = [f"    const double {sym} = {sp.ccode(ex)};" for sym, ex in repl]
    lines += [f"    {nm} = {sp.ccode(ex)};" for nm, ex in zip(names, red)]
    scal = ["s0", "s1", "s2", "v0", "v1", "v2", "G0", "G1", "G2", "gB0", "gB1", "gB2",
            "gP0", "gP1", "gP2", "ab0", "ab1", "ab2", "bb0", "bb1", "bb2",
            "Phi", "S0", "U", "mi", "m0", "eps", "eps2", "ic2", "gA", "gC"]
    outv = ["s_b", "v_b", "G_b", "W_b", "gB_b", "gP_b"]
    outs_s = ["Phi_b", "S0_b", "U_b", "m0_b", "gA_b", "gC_b"]
    sig = (", ".join(f"double {x}" for x in scal) + ",\n    " +
           ", ".join(f"double {x}[3]" for x in outv) + ",\n    " +
           ", ".join(f"double &{x}" for x in outs_s))
    body = "\n".join(lines)
    src = f'''// pn_finish_vjp_gen.cuh -- GENERATED by gen_finish_vjp.py from the finishing kernel's
// formulas; regenerate instead of editing.
//
// Adjoint of the per-star closed forms: given ab = abar_i and bb = abar_0, the gradients of
// L_i = ab . a_i + ic2 * bb . bh_i with respect to the star's s, v, pair sums (G, Phi, S0, U,
// W), the BH mass m0 and the global sums (gA = A1, gC = C, gB = B3, gP = P).
#pragma once

namespace pn {{

__device__ __forceinline__ double pn_ipow(double x, int n) {{
    double r = 1.0;
    const bool inv = n < 0;
    for (int k = 0; k < (inv ? -n : n); ++k) r *= x;
    return inv ? 1.0 / r : r;
}}
__device__ __forceinline__ double pn_ipow(double x, double n) {{
    // sympy writes R = (q + eps2)^(-1/2) powers as pow(.., -1/2), -3/2, ...
    return pow(x, n);
}}

__device__ __forceinline__ void finish_vjp_gen(
    {sig}) {{
#define pow(a, b) pn_ipow((double)(a), (b))
{body}
#undef pow
}}

}}  // namespace pn
'''
    with open(OUT, "w") as f:
        f.write(src)
    print("wrote", OUT, len(repl), "common subexpressions")


if __name__ == "__main__":
    main()
