"""Generates the golden element and assembly fixtures that pin the CPU oracle.

The reference ships no tests, fixtures or golden vectors, and it cannot be run here
(Julia is absent; its C++ side needs Eigen, whose submodule is empty).  These fixtures
are derived independently of the oracle, in exact rational arithmetic (sympy and
fractions), from the formulas the reference states:

* P1 tetrahedron / triangle stiffness and mass on the unit right simplex
  (src/FEM3D.jl:59-76, 466-492; src/FEM2D.jl:48-76, 139-161);
* P2 stiffness with the reference's equal-weight rule at the element nodes
  (src/FEM3D.jl:344-364 over 10 nodes /10; src/FEM2D.jl:95-107 over 6 nodes /6);
* P2 mass with the reference's Gauss tables and weight scaling
  (src/FEM3D.jl:494-561 with GaussQuadrature3D(4), including the linear-part-only
  basis evaluation of :529-531; src/FEM2D.jl:163-229 with GaussQuadrature2D(4));
* the global stiffness of the unjittered 2x2x2-cell Kuhn mesh, assembled by summing
  element matrices into a dictionary keyed by (row, column).

Run:  python tests/golden/make_golden.py   (writes the JSON files beside it)
"""
from __future__ import annotations

import itertools
import json
import os
from fractions import Fraction

import sympy as S

HERE = os.path.dirname(os.path.abspath(__file__))

X, Y, Z = S.symbols("x y z")


def p1_grads_3d(P):
    """Gradients of the P1 basis on the tetrahedron with vertices P (rational)."""
    M = S.Matrix([[1, *P[a]] for a in range(4)])
    C = M.inv()  # columns: coefficients (a, b, c, d) of each basis function
    return [[C[1, a], C[2, a], C[3, a]] for a in range(4)], abs(M.det()) / 6


def p1_grads_2d(P):
    M = S.Matrix([[1, *P[a]] for a in range(3)])
    C = M.inv()
    return [[C[1, a], C[2, a]] for a in range(3)], abs(M.det()) / 2


def basis_p2_3d(nodes):
    mons = [S.Integer(1), X, Y, Z, X * X, X * Y, X * Z, Y * Y, Y * Z, Z * Z]
    V = S.Matrix([[m.subs({X: n[0], Y: n[1], Z: n[2]}) for m in mons] for n in nodes])
    Cf = V.inv()
    return [sum(Cf[c, a] * mons[c] for c in range(10)) for a in range(10)], [[Cf[c, a] for c in range(10)] for a in range(10)]


def basis_p2_2d(nodes):
    mons = [S.Integer(1), X, Y, X * X, X * Y, Y * Y]
    V = S.Matrix([[m.subs({X: n[0], Y: n[1]}) for m in mons] for n in nodes])
    Cf = V.inv()
    return [sum(Cf[c, a] * mons[c] for c in range(6)) for a in range(6)], [[Cf[c, a] for c in range(6)] for a in range(6)]


def tofloat(M):
    return [[float(v) for v in row] for row in M]


# Gauss tables of src/FEM3D.jl:712-745 and src/FEM2D.jl:485-497, as the decimal
# strings printed there (exact rationals of those decimals).
GQ3_P = ["0.2500000000000000 0.2500000000000000 0.2500000000000000", "0.0000000000000000 0.3333333333333333 0.3333333333333333",
         "0.3333333333333333 0.3333333333333333 0.3333333333333333", "0.3333333333333333 0.3333333333333333 0.0000000000000000",
         "0.3333333333333333 0.0000000000000000 0.3333333333333333", "0.7272727272727273 0.0909090909090909 0.0909090909090909",
         "0.0909090909090909 0.0909090909090909 0.0909090909090909", "0.0909090909090909 0.0909090909090909 0.7272727272727273",
         "0.0909090909090909 0.7272727272727273 0.0909090909090909", "0.4334498464263357 0.0665501535736643 0.0665501535736643",
         "0.0665501535736643 0.4334498464263357 0.0665501535736643", "0.0665501535736643 0.0665501535736643 0.4334498464263357",
         "0.0665501535736643 0.4334498464263357 0.4334498464263357", "0.4334498464263357 0.0665501535736643 0.4334498464263357",
         "0.4334498464263357 0.4334498464263357 0.0665501535736643"]
GQ3_W = ["0.1817020685825351"] + ["0.0361607142857143"] * 4 + ["0.0698714945161738"] * 4 + ["0.0656948493683187"] * 6
GQ2_P = ["0.445948490915965 0.445948490915965", "0.445948490915965 0.108103018168070", "0.108103018168070 0.445948490915965",
         "0.091576213509771 0.091576213509771", "0.091576213509771 0.816847572980459", "0.816847572980459 0.091576213509771"]
GQ2_W = ["0.223381589678011"] * 3 + ["0.109951743655322"] * 3


def element_fixtures():
    out = {}
    P3 = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
    g, VE = p1_grads_3d(P3)
    K = [[VE * sum(g[a][d] * g[b][d] for d in range(3)) for b in range(4)] for a in range(4)]
    M = [[VE * S.Rational(2 if a == b else 1, 20) for b in range(4)] for a in range(4)]
    out["tet4_unit"] = {"p": P3, "K": tofloat(K), "M": tofloat(M), "VE": float(VE)}
    P2 = [(0, 0), (1, 0), (0, 1)]
    g2, A = p1_grads_2d(P2)
    K2 = [[A * sum(g2[a][d] * g2[b][d] for d in range(2)) for b in range(3)] for a in range(3)]
    M2 = [[A * S.Rational(2 if a == b else 1, 12) for b in range(3)] for a in range(3)]
    out["tri3_unit"] = {"p": P2, "K": tofloat(K2), "M": tofloat(M2), "VE": float(A)}

    # P2 tetrahedron on the unit simplex, Gmsh node order (edges 01, 12, 20, 30, 32, 31)
    V = [S.Matrix(v) for v in P3]
    edges = [(0, 1), (1, 2), (2, 0), (3, 0), (3, 2), (3, 1)]
    nodes = [tuple(v) for v in V] + [tuple((V[a] + V[b]) / 2) for a, b in edges]
    phis, coef = basis_p2_3d(nodes)
    grads = [[S.diff(f, v) for v in (X, Y, Z)] for f in phis]
    VE10 = S.Rational(1, 6)
    Kp2 = [[S.Rational(0)] * 10 for _ in range(10)]
    for n in nodes:
        sub = {X: n[0], Y: n[1], Z: n[2]}
        gv = [[gr[d].subs(sub) for d in range(3)] for gr in grads]
        for i in range(10):
            for j in range(10):
                Kp2[i][j] += sum(gv[i][d] * gv[j][d] for d in range(3))
    Kp2 = [[v / 10 * VE10 for v in row] for row in Kp2]
    pts = [[S.Rational(s) for s in line.split()] for line in GQ3_P]
    wts = [S.Rational(w) / 6 for w in GQ3_W]

    def p2_mass(full):
        Mm = [[S.Rational(0)] * 10 for _ in range(10)]
        for (xi, eta, ze), w in zip(pts, wts):
            x, y, z = xi, eta, ze   # unit simplex: physical = reference coordinates
            vals = []
            for a in range(10):
                c = coef[a]
                v = c[0] + c[1] * x + c[2] * y + c[3] * z
                if full:
                    v += c[4] * x * x + c[5] * x * y + c[6] * x * z + c[7] * y * y + c[8] * y * z + c[9] * z * z
                vals.append(v)
            for i in range(10):
                for j in range(10):
                    Mm[i][j] += w * VE10 * vals[i] * vals[j]
        return Mm

    out["tet10_unit"] = {"p": [[float(c) for c in n] for n in nodes], "K": tofloat(Kp2),
                         "M_full": tofloat(p2_mass(True)), "M_linear_part": tofloat(p2_mass(False)),
                         "VE": float(VE10)}

    # P2 triangle, Gmsh order (edges 01, 12, 20)
    W = [S.Matrix(v) for v in P2]
    nodes2 = [tuple(v) for v in W] + [tuple((W[a] + W[b]) / 2) for a, b in [(0, 1), (1, 2), (2, 0)]]
    phis2, coef2 = basis_p2_2d(nodes2)
    grads2 = [[S.diff(f, v) for v in (X, Y)] for f in phis2]
    A6 = S.Rational(1, 2)
    Kt6 = [[S.Rational(0)] * 6 for _ in range(6)]
    for n in nodes2:
        sub = {X: n[0], Y: n[1]}
        gv = [[gr[d].subs(sub) for d in range(2)] for gr in grads2]
        for i in range(6):
            for j in range(6):
                Kt6[i][j] += gv[i][0] * gv[j][0] + gv[i][1] * gv[j][1]
    Kt6 = [[v / 6 * A6 for v in row] for row in Kt6]
    Mt6 = [[S.Rational(0)] * 6 for _ in range(6)]
    for line, w in zip(GQ2_P, GQ2_W):
        xi, eta = [S.Rational(s) for s in line.split()]
        vals = [phis2[a].subs({X: xi, Y: eta}) for a in range(6)]
        for i in range(6):
            for j in range(6):
                Mt6[i][j] += S.Rational(w) * A6 * vals[i] * vals[j]
    out["tri6_unit"] = {"p": [[float(c) for c in n] for n in nodes2], "K": tofloat(Kt6), "M": tofloat(Mt6),
                        "VE": float(A6)}
    return out


def kuhn2_stiffness():
    """Exact global stiffness of the unjittered 2x2x2-cell Kuhn mesh of [-5,5]^3."""
    n, N, L = 2, 3, 5
    h = Fraction(2 * L, n)
    coord = lambda i: -L + i * h  # noqa: E731
    p = {}
    for k in range(N):
        for j in range(N):
            for i in range(N):
                p[i + N * (j + N * k)] = (coord(i), coord(j), coord(k))
    tets = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                for perm in itertools.permutations(range(3)):
                    cur = [i, j, k]
                    vs = [cur[0] + N * (cur[1] + N * cur[2])]
                    for ax in perm:
                        cur = cur.copy()
                        cur[ax] += 1
                        vs.append(cur[0] + N * (cur[1] + N * cur[2]))
                    tets.append(vs)
    acc = {}
    for vs in tets:
        P = [tuple(S.Rational(c.numerator, c.denominator) for c in p[v]) for v in vs]
        g, VE = p1_grads_3d(P)
        for a in range(4):
            for b in range(4):
                val = VE * sum(g[a][d] * g[b][d] for d in range(3))
                acc[(vs[a], vs[b])] = acc.get((vs[a], vs[b]), 0) + val
    nv = N ** 3
    colptr, rowval, data = [0], [], []
    for c in range(nv):
        rows = sorted(r for (r, cc) in acc if cc == c)
        for r in rows:
            rowval.append(r)
            data.append(float(acc[(r, c)]))
        colptr.append(len(rowval))
    return {"cells": n, "nv": nv, "colptr": colptr, "rowval": rowval, "data": data,
            "exact_zero_entries": sum(1 for v in acc.values() if v == 0)}


if __name__ == "__main__":
    with open(os.path.join(HERE, "element_matrices.json"), "w") as f:
        json.dump(element_fixtures(), f, indent=1)
    with open(os.path.join(HERE, "kuhn2_stiffness.json"), "w") as f:
        json.dump(kuhn2_stiffness(), f)
    print("written")
