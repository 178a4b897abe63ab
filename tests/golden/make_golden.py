"""Generates tests/golden/operators_exact.json: exact rational golden vectors.

The reference (Julia) cannot run on these machines, so the golden vectors are computed
from the reference's own dense definitions in exact rational arithmetic (fractions):
  - Dr/Ds/Dt from getindex/get_coeff   (src/BernsteinDerivativeMatrix_3D.jl:61-94)
  - ElevationMatrix                    (src/ElevationMatrix.jl:17-24)
  - face lift [L0; l_i E'...L0]        (test/runtests.jl:34-40)
  - full lift M^{-1}[M^1|M^2|M^3|M^4]  (the definition get_bernstein_lift computes,
                                        src/utility.jl:157-180, with exact mass matrices)
applied to fixed rational inputs. Values are stored as "p/q" strings and as the nearest
double. Run: python tests/golden/make_golden.py
"""
import json
import os
import sys
from fractions import Fraction

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import dense  # noqa: E402


def rational_input(n, salt):
    return [Fraction(((m * 37 + 11 * salt + 5) % 23) - 11, 7 + (m % 3)) for m in range(n)]


def matvec(M, x):
    return [sum((a * b for a, b in zip(row, x)), Fraction(0)) for row in M]


def enc(v):
    return {"exact": [f"{q.numerator}/{q.denominator}" for q in v], "float": [float(q) for q in v]}


def main():
    out = {"description": __doc__.strip().splitlines()[0], "cases": []}
    F = Fraction
    for N in range(1, 7):
        Np = (N + 1) * (N + 2) * (N + 3) // 6
        x = rational_input(Np, N)
        for axis, name in enumerate("rst"):
            D = dense.deriv_dense(N, axis, num=F)
            out["cases"].append({"op": f"D{name}", "N": N, "x": enc(x), "y": enc(matvec(D, x))})
    for N in range(1, 8):
        Nfp = (N + 1) * (N + 2) // 2
        x = rational_input(Nfp, 100 + N)
        E = dense.elevation_dense(N + 1, num=F)
        out["cases"].append({"op": "elevation", "N": N, "x": enc(x), "y": enc(matvec(E, x))})
        Et = [list(r) for r in zip(*dense.elevation_dense(N, num=F))]  # reduction_multiply! = ElevationMatrix{N}^T
        out["cases"].append({"op": "reduction", "N": N, "x": enc(x),
                             "y": enc(matvec(Et, x))})
    for N in range(1, 6):
        Nfp = (N + 1) * (N + 2) // 2
        x = rational_input(Nfp, 200 + N)
        out["cases"].append({"op": "face_lift", "N": N, "x": enc(x),
                             "y": enc(matvec(dense.face_lift_dense(N, num=F), x))})
    for N in range(1, 5):
        Nfp = (N + 1) * (N + 2) // 2
        x = rational_input(4 * Nfp, 300 + N)
        L = dense.lift_from_mass(N, num=F)
        out["cases"].append({"op": "lift", "N": N, "x": enc(x), "y": enc(matvec(L, x))})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "operators_exact.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=None, separators=(",", ":"))
    print(path, len(out["cases"]), "cases")


if __name__ == "__main__":
    main()
