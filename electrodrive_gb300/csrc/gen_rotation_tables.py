"""Generate rotation_tables.h: the fixed quarter-turn rotation matrices of the
rotation-based M2L, exact.

The solid harmonics of the library (harmonics.cuh),
    R_n^m(v) = |v|^n P_n^m(cos t) e^{i m phi} / (n + m)!,
are polynomials in (x, y, z) with complex rational coefficients.  A rotation
Q that permutes the axes (here the quarter turns about x, Q v = (x, -z, y)
and its inverse) maps each R_n^m(Q v) into span{R_n^m'(v)} with complex
rational coefficients T^n_{m m'}: R_n^m(Q v) = sum_m' T^n_{m m'} R_n^m'(v).
They are found here by exact linear algebra (sympy rationals).

The kernels keep a degree-n block of coefficients X_0..X_n (m >= 0; X_{-m} =
(-1)^m conj(X_m) for real fields) as the real vector
[Re X_0, Re X_1, Im X_1, ..., Re X_n, Im X_n].  In that basis every linear
map that keeps the symmetry is a real (2n+1) x (2n+1) matrix.  The tables are:

  FWD_P = realify(conj(T(Qp)))   multipoles, quarter turn +pi/2 about x
  FWD_M = realify(conj(T(Qm)))   multipoles, -pi/2
  BWD_P = realify(T(Qp)^T)       locals
  BWD_M = realify(T(Qm)^T)

With R_y(b) = Q_m R_z(b) Q_p and R_z acting as e^{i m a}, a rotation about y
costs two fixed sparse matrices and one diagonal of phases.

    python electrodrive_gb300/csrc/gen_rotation_tables.py [pmax]   (default 8)
"""
from __future__ import annotations

import os
import sys

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))


def solid_harmonics(p, x, y, z):
    """R_n^m for 0 <= m <= n <= p as sympy expressions (the library's recurrences)."""
    R = {(0, 0): sp.Integer(1)}
    r2 = x * x + y * y + z * z
    for m in range(1, p + 1):
        R[(m, m)] = sp.expand(-(x + sp.I * y) / (2 * m) * R[(m - 1, m - 1)])
    for m in range(0, p + 1):
        for n in range(m + 1, p + 1):
            a = R[(n - 1, m)]
            b = R[(n - 2, m)] if n - 2 >= m else 0
            R[(n, m)] = sp.expand(((2 * n - 1) * z * a - r2 * b) / ((n + m) * (n - m)))
    return R


def harmonic(R, n, m):
    if m >= 0:
        return R[(n, m)]
    return sp.expand((-1) ** (-m) * sp.conjugate(R[(n, -m)]))


def rotation_T(R, n, subs, x, y, z):
    """T[m][m'] with R_n^m(Qv) = sum_m' T[m][m'] R_n^m'(v), m, m' in -n..n."""
    basis = [sp.Poly(harmonic(R, n, mp), x, y, z) for mp in range(-n, n + 1)]
    monos = sorted({mono for b in basis for mono in b.monoms()})
    A = sp.Matrix([[b.coeff_monomial(mono) for b in basis] for mono in monos])
    T = []
    for m in range(-n, n + 1):
        target = sp.Poly(sp.expand(harmonic(R, n, m).subs(subs, simultaneous=True)), x, y, z)
        rhs = sp.Matrix([target.coeff_monomial(mono) for mono in monos])
        sol = A.solve_least_squares(rhs) if A.shape[0] != A.shape[1] else A.solve(rhs)
        T.append([sp.nsimplify(sp.simplify(v)) for v in sol])
    return T  # T[m + n][m' + n]


def realify(M, n):
    """Real matrix of x -> M @ full(x) on the real vector [a0, a1, b1, ...]."""
    size = 2 * n + 1
    W = [[sp.Integer(0)] * size for _ in range(size)]
    for j in range(size):
        # basis vector j -> complex coefficients X_0..X_n
        X = [sp.Integer(0)] * (n + 1)
        if j == 0:
            X[0] = sp.Integer(1)
        else:
            m = (j + 1) // 2
            X[m] = sp.Integer(1) if j % 2 == 1 else sp.I
        full = [(-1) ** (-m) * sp.conjugate(X[-m]) if m < 0 else X[m] for m in range(-n, n + 1)]
        y = [sp.expand(sum(M[i][k] * full[k] for k in range(size))) for i in range(size)]
        ym = y[n:]  # outputs m = 0..n
        col = [sp.re(ym[0])]
        for m in range(1, n + 1):
            col += [sp.re(ym[m]), sp.im(ym[m])]
        for i in range(size):
            W[i][j] = sp.nsimplify(col[i])
    return W


def main(pmax=8):
    x, y, z = sp.symbols("x y z", real=True)
    R = solid_harmonics(pmax, x, y, z)
    qp = {x: x, y: -z, z: y}   # quarter turn +pi/2 about x
    qm = {x: x, y: z, z: -y}   # -pi/2
    tables = {"FWD_P": [], "FWD_M": [], "BWD_P": [], "BWD_M": []}
    for n in range(pmax + 1):
        Tp = rotation_T(R, n, qp, x, y, z)
        Tm = rotation_T(R, n, qm, x, y, z)
        conj = lambda M: [[sp.conjugate(v) for v in row] for row in M]
        transp = lambda M: [list(r) for r in zip(*M)]
        tables["FWD_P"].append(realify(conj(Tp), n))
        tables["FWD_M"].append(realify(conj(Tm), n))
        tables["BWD_P"].append(realify(transp(Tp), n))
        tables["BWD_M"].append(realify(transp(Tm), n))
        print(f"degree {n} done", file=sys.stderr)
    out = [
        "// Generated by gen_rotation_tables.py: exact quarter-turn rotation matrices",
        "// of the solid harmonics in the real block basis [Re X0, Re X1, Im X1, ...],",
        "// degree n block of size (2n+1)^2 at offset kRotOff[n], row-major.",
        "#pragma once",
        "",
        "namespace edfmm {",
        "",
        f"constexpr int kRotPMax = {pmax};",
    ]
    offs, o = [], 0
    for n in range(pmax + 1):
        offs.append(o)
        o += (2 * n + 1) ** 2
    out.append("constexpr int kRotOff[%d] = {%s};" % (pmax + 2, ", ".join(str(v) for v in offs + [o])))
    for name, blocks in tables.items():
        vals = []
        for n, W in enumerate(blocks):
            for row in W:
                for v in row:
                    vals.append(repr(float(sp.N(v, 30))))
        out.append(f"constexpr double kRot{name.title().replace('_', '')}[{o}] = {{")
        for i in range(0, len(vals), 6):
            out.append("    " + ", ".join(vals[i:i + 6]) + ",")
        out.append("};")
    out += ["", "}  // namespace edfmm", ""]
    with open(os.path.join(HERE, "rotation_tables.h"), "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 8)
