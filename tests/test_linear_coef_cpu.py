"""The generated coefficient tables of the gate's linear path (hos_linear_coef.cuh) are up to date
and equal the full-stencil polynomials of the WENO-AO formulas in hos_weno.cuh (the reference's
polynomials, src/reconstruction.cpp): each formula is evaluated at unit stencils with the DF
factor 1 and unit spacing, which gives its coefficient per stencil cell."""
import math
import re
import subprocess
import sys
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "high-order-solver_gb300" / "csrc"
WENO = (CSRC / "hos_weno.cuh").read_text()
COEF = (CSRC / "hos_linear_coef.cuh").read_text()


def _table(kind, order, name):
    m = re.search(rf"struct {kind}<{order}> \{{.*?{name}\(int p, int k\) \{{\s*constexpr double c\[\d+\]\[\d+\] = (\{{.*?\}});",
                  COEF, re.S)
    return eval(m.group(1).replace("{", "[").replace("}", "]"))


def _body(fn):
    i = WENO.index(fn)
    return WENO[i:WENO.index("\n}\n", i)]


def _stmts(text, lhs):
    return [m.group(1) for m in re.finditer(re.escape(lhs) + r" = (.*?);", text, re.S)]


def _coeffs(expr, n, extra=None):
    r = n // 2
    out = []
    for k in range(n):
        env = dict(T=float, ih=1.0, df=[1.0] * 6)
        for i in range(n):
            off = i - r
            env["w0" if off == 0 else (f"wn{-off}" if off < 0 else f"wp{off}")] = 1.0 if i == k else 0.0
        env.update(extra or {})
        out.append(eval(expr.replace("\n", " "), {}, env))
    return out


def test_header_is_generated_from_the_script():
    pytest.importorskip("sympy")
    r = subprocess.run([sys.executable, str(CSRC / "gen_linear_coef.py"), "--check"])
    assert r.returncode == 0, "hos_linear_coef.cuh differs from gen_linear_coef.py's output"


@pytest.mark.parametrize("order,top", [(5, 3), (7, 4), (9, 5)])
def test_normal_tables_match_the_weno_formulas(order, top):
    nb = _body("normal_face")
    vals, ders = _stmts(nb, f"p[{top}]"), _stmts(nb, f"px[{top}]")
    V, D = _table("Normal", order, "V"), _table("Normal", order, "D")
    for side in range(2):
        assert max(abs(a - b) for a, b in zip(_coeffs(vals[side], order), V[side])) < 1e-14
        assert max(abs(a - b) for a, b in zip(_coeffs(ders[side], order), D[side])) < 1e-14


@pytest.mark.parametrize("order,top,q,npts", [(5, 3, math.sqrt(3), 2), (7, 4, math.sqrt(15), 3)])
def test_tangent_tables_match_the_weno_formulas(order, top, q, npts):
    seg = _body("tangent_point")
    seg = seg[seg.index(f"ORDER == {order}"):]
    vals, ders = _stmts(seg, f"p[{top}]")[:npts], _stmts(seg, f"px[{top}]")[:npts]
    V, D = _table("Tangent", order, "V"), _table("Tangent", order, "D")
    for ig in range(npts):
        assert max(abs(a - b) for a, b in zip(_coeffs(vals[ig], order, {"q": q}), V[ig])) < 1e-14
        assert max(abs(a - b) for a, b in zip(_coeffs(ders[ig], order, {"q": q}), D[ig])) < 1e-14


def test_tangent_table_order9_matches_the_polynomial_family():
    # the 9th-order family is written as a polynomial in x on the segment [-1, 0] (Lobatto
    # abscissae x = -1, 0, -1/2 -+ sqrt(5)/10): collect its coefficients the same way
    tb = _body("tangent_point")
    seg = tb[tb.index("T a9, b9, c9"):tb.index("const T x7 = x6 * x")]
    seg = seg.replace("T a9, b9, c9, d9, e9, f9, g9, h9, i9;", "").replace(";", "\n").replace("\n        ", "\n")
    names = ["wn4", "wn3", "wn2", "wn1", "w0", "wp1", "wp2", "wp3", "wp4"]
    V, D = _table("Tangent", 9, "V"), _table("Tangent", 9, "D")
    r5 = math.sqrt(5.0)
    for ig, x in enumerate((-1.0, 0.0, -0.5 - r5 / 10, -0.5 + r5 / 10)):
        for k in range(9):
            env = dict(T=float, **{nm: 1.0 if i == k else 0.0 for i, nm in enumerate(names)})
            exec(seg, {}, env)
            c = [env[f"{ch}9"] for ch in "abcdefghi"]
            val = sum(c[m] * x**m for m in range(9))
            der = sum(m * c[m] * x ** (m - 1) for m in range(1, 9))
            assert abs(val - V[ig][k]) < 1e-13
            assert abs(der - D[ig][k]) < 1e-13
