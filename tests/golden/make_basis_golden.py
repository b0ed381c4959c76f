"""Generates tests/golden/basis_golden.npz from the reference's own
src/basis_functions.h, compiled unmodified by oracle/Makefile into
oracle/_ref/libref_basis.so.  Run where the Karamelo tree is available:

    make -C oracle ref && python tests/golden/make_basis_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle  # noqa: E402


def main():
    L = oracle.ref_basis_lib()
    if L is None:
        raise SystemExit("oracle/_ref/libref_basis.so is missing: build it with `make -C oracle ref`")
    # r on a grid that hits every branch boundary exactly, plus interior points
    r = np.unique(np.concatenate([np.linspace(-2.5, 2.5, 1001), np.array([-2, -1.5, -1, -0.5, 0, 0.5, 1, 1.5, 2]),
                                  np.array([-1e-12, 1e-12, 0.999999999, -0.999999999, 1.999999999])]))
    out = {"r": r}
    icell = 2.5
    for basis, ntypes in ((0, [0]), (1, [-2, -1, 0, 1, 2]), (2, [0, 1]), (3, [-2, -1, 0, 1, 2])):
        for nt in ntypes:
            for kind in (0, 1):
                out[f"b{basis}_n{nt}_k{kind}"] = np.array([L.ref_basis(basis, kind, float(x), nt, icell) for x in r])
    out["icellsize"] = np.array(icell)
    np.savez_compressed(os.path.join(HERE, "basis_golden.npz"), **out)
    print("wrote", len(out) - 2, "golden vectors over", r.size, "points")


if __name__ == "__main__":
    main()
