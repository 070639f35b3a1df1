"""Regenerate tests/golden/tominec_fitted.npz from the reference's own test fixtures.

The reference's regression tests (test/poisson_test.jl, test/hyperviscosity_test.jl)
read Tominec's fitted node sets and index sets from CSV files under test/data/.
This script converts exactly those files, unmodified, into one compressed .npz so
that the parity tests can run where the reference checkout is absent.

Usage:  python tests/golden/make_golden.py path/to/RadialBasisFiniteDifferences.jl
"""
import os
import sys

import numpy as np


def main(ref_root):
    data = os.path.join(ref_root, "test", "data")

    def csv(name, dtype=np.float64):
        return np.loadtxt(os.path.join(data, name), delimiter=",", dtype=dtype, ndmin=1)

    out = dict(
        # test/poisson_test.jl:14-15,19-22: X = x_nodes_fitted (N=2000), Y = y_nodes_fitted
        x_nodes=csv("x_nodes_fitted.csv").reshape(-1, 2),
        y_nodes=csv("y_nodes_fitted.csv").reshape(-1, 2),
        # test/poisson_test.jl:28-32: 1-based index sets and normals (column 3 = normal component)
        y_idx_in=csv("Y_idx_in.csv", np.int64),
        y_idx_dirichlet=csv("Y_idx_dirichlet.csv", np.int64),
        y_idx_neumann=csv("Y_idx_neumann.csv", np.int64),
        x_normals=csv("x_normals.csv").reshape(-1, 3),
        y_normals=csv("y_normals.csv").reshape(-1, 3),
    )
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tominec_fitted.npz")
    np.savez_compressed(dst, **out)
    for k, v in out.items():
        print(f"{k}: {v.shape} {v.dtype}")
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py path/to/RadialBasisFiniteDifferences.jl (the reference checkout)")
    main(sys.argv[1])
