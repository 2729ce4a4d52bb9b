"""Writes tests/golden/golden.json: known-answer vectors that pin the CPU
restatement (oracle/) of the reference.  No value here comes from running
the oracle or the GPU library; each is a closed form or a hand derivation.

Run:  python tests/golden/make_golden.py
"""
import json
import os
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))


def dot_kat(n):
    # src/BenchMark.f:444-485: x(i) = i, y(i) = 2i  ->  x.y = 2 n(n+1)(2n+1)/6
    return 2 * n * (n + 1) * (2 * n + 1) // 6


def main():
    g = {}
    g["dot_kat"] = {str(n): dot_kat(n) for n in (1, 2, 3, 4, 5, 7, 100, 1000, 4097, 100000)}

    # 2x2 quad mesh, nodes row by row (1..9), cells (0,0)=1 (1,0)=2 (0,1)=3
    # (1,1)=4, each cell (n00,n10,n11,n01).  Sides: 1 bottom, 2 right, 3 top,
    # 4 left.  Hand-derived face neighbours (src/Adjacency.f:95-189):
    g["quad2x2"] = {
        "ix": [[1, 2, 5, 4], [2, 3, 6, 5], [4, 5, 8, 7], [5, 6, 9, 8]],
        "nnode": 9,
        "nelcon": [[-1, 2, 3, -1], [-1, -1, 4, 1], [1, 4, -1, -1], [2, -1, -1, 3]],
        # RCM by hand (src/Reord.f): fnroot from 1 -> last level {4}, the
        # single-node last level makes 4 the root (nunlvl = nlvl = 3 stops);
        # degrees all 2; Cuthill-McKee from 4: 4, 2, 3, 1; reversed
        # perm = 1, 3, 2, 4; num(perm(i)) = i.
        "num": [1, 3, 2, 4],
    }
    # 4x1 strip of quads: a path graph 1-2-3-4.  rootls from 1 gives 4
    # levels = ccsize, so fnroot keeps root 1; Cuthill-McKee 1,2,3,4;
    # reversed 4,3,2,1; num = [4,3,2,1].
    g["strip4"] = {
        "ix": [[1, 2, 7, 6], [2, 3, 8, 7], [3, 4, 9, 8], [4, 5, 10, 9]],
        "nnode": 10,
        "nelcon": [[-1, 2, -1, -1], [-1, 3, -1, 1], [-1, 4, -1, 2], [-1, -1, -1, 3]],
        "num": [4, 3, 2, 1],
    }
    # 2x2 SPD system for the Krylov solvers: A = [[4,-1],[-1,3]] stored as
    # CSRD (the stored off-diagonal values are A_ij themselves: au = [-1, -1],
    # i.e. the assembly's negated face coefficients), b = [1, 2].
    # Exact solution A^-1 b = [5/11, 9/11].  Jacobi-PCG / BiCGSTAB / GMRES
    # reach it in 2 steps in exact arithmetic (2 distinct eigenvalues).
    A = [[Fraction(4), Fraction(-1)], [Fraction(-1), Fraction(3)]]
    b = [Fraction(1), Fraction(2)]
    det = A[0][0] * A[1][1] - A[0][1] * A[1][0]
    x = [(A[1][1] * b[0] - A[0][1] * b[1]) / det, (A[0][0] * b[1] - A[1][0] * b[0]) / det]
    g["spd2"] = {"ad": [4.0, 3.0], "ia": [1, 2, 3], "ja": [2, 1], "au": [-1.0, -1.0],
                 "b": [1.0, 2.0], "x": [float(v) for v in x],
                 "x_fraction": [str(v) for v in x]}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
