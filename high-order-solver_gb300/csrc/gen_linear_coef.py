"""Generate hos_linear_coef.cuh: the coefficients of the full-stencil (linear-weight)
reconstruction that the learned gate's linear path evaluates.

The top candidate of WENO-AO(ORDER) is the polynomial P of degree ORDER - 1 whose averages over
the ORDER stencil cells equal the cell values s_k (cells of unit width centred at k - ORDER // 2).
Its value and slope at a point xi of the centre cell are linear in s:
    P(xi) = sum_k V[k] s_k,   h P'(xi) = sum_k D[k] s_k.
The reference writes these polynomials term by term with the Gauss point folded into each
coefficient (src/reconstruction.cpp: the normal faces of WENO5/7/9-AO, :480-657, :750-974,
:1072-1364; the tangential Gauss-point forms, :2751-2836, :3021-3174, :3557-3609); collected
per stencil cell they are these tables (tests/test_linear_coef_cpu.py evaluates the device
formulas of hos_weno.cuh at unit stencils and compares).

Points: the normal faces xi = -1/2 (left, side 0) and +1/2 (right, side 1); the tangential Gauss
points of gausspoint 2 / 3 / 4 (SetGuassPoint: Gauss-Legendre 2 and 3, Lobatto 4) in the order
the reference numbers them: WENO5 -sqrt(3)/6, +sqrt(3)/6; WENO7 0, -sqrt(15)/10, +sqrt(15)/10;
WENO9 -1/2, +1/2, -sqrt(5)/10, +sqrt(5)/10.

    python gen_linear_coef.py            # rewrite hos_linear_coef.cuh beside this file
    python gen_linear_coef.py --check    # exit 1 if the file differs from what would be written
"""
from __future__ import annotations

import sys
from pathlib import Path

import sympy as sp

OUT = Path(__file__).resolve().parent / "hos_linear_coef.cuh"
XI = sp.symbols("xi")
HALF = sp.Rational(1, 2)
TANGENT_POINTS = {
    5: (-sp.sqrt(3) / 6, sp.sqrt(3) / 6),
    7: (sp.Integer(0), -sp.sqrt(15) / 10, sp.sqrt(15) / 10),
    9: (-HALF, HALF, -sp.sqrt(5) / 10, sp.sqrt(5) / 10),
}


def polynomial(n: int):
    """P(xi) with cell averages s_0 .. s_{n-1} over [k - r - 1/2, k - r + 1/2]; returns (P, s)."""
    r = n // 2
    c = sp.symbols(f"c0:{n}")
    s = sp.symbols(f"s0:{n}")
    p = sum(c[i] * XI**i for i in range(n))
    eqs = [sp.integrate(p, (XI, k - r - HALF, k - r + HALF)) - s[k] for k in range(n)]
    return p.subs(sp.solve(eqs, c)), s


def table(n: int, points) -> tuple[list[list[float]], list[list[float]]]:
    p, s = polynomial(n)
    dp = sp.diff(p, XI)
    vals, ders = [], []
    for x in points:
        pv, dv = sp.expand(p.subs(XI, x)), sp.expand(dp.subs(XI, x))
        vals.append([float(sp.N(pv.coeff(s[k]), 40)) for k in range(n)])
        ders.append([float(sp.N(dv.coeff(s[k]), 40)) for k in range(n)])
    return vals, ders


def fmt(rows: list[list[float]]) -> str:
    return "{" + ", ".join("{" + ", ".join(repr(v) for v in row) + "}" for row in rows) + "}"


def render() -> str:
    out = [
        "// hos_linear_coef.cuh -- GENERATED by gen_linear_coef.py (do not edit): coefficients of the",
        "// full-stencil polynomial of WENO-AO(ORDER), the reconstruction the learned gate's linear path",
        "// evaluates.  Value = sum_k V(p, k) s[k], slope = ih * sum_k D(p, k) s[k] for the stencil",
        "// s[0 .. ORDER-1] centred on the cell; p = side (normal faces: 0 left, 1 right) or Gauss point",
        "// (tangential, the reference's numbering).",
        "#pragma once",
        "",
        "namespace hos {",
        "namespace lin {",
        "",
        "template <int ORDER> struct Normal;",
        "template <int ORDER> struct Tangent;",
    ]
    for n in (5, 7, 9):
        nv, nd = table(n, (-HALF, HALF))
        tv, td = table(n, TANGENT_POINTS[n])
        out += [""]
        for kind, v, d in (("Normal", nv, nd), ("Tangent", tv, td)):
            out.append(f"template <> struct {kind}<{n}> {{")
            for name, rows in (("V", v), ("D", d)):
                out += [
                    f"    __host__ __device__ static constexpr double {name}(int p, int k) {{",
                    f"        constexpr double c[{len(rows)}][{n}] = {fmt(rows)};",
                    "        return c[p][k];",
                    "    }",
                ]
            out.append("};")
    out += ["", "}  // namespace lin", "}  // namespace hos", ""]
    return "\n".join(out)


if __name__ == "__main__":
    text = render()
    if "--check" in sys.argv:
        sys.exit(0 if OUT.exists() and OUT.read_text() == text else 1)
    OUT.write_text(text)
    print(f"wrote {OUT}")
