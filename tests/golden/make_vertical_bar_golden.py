"""Generates tests/golden/vertical_bar_golden.npz from the reference's own
published runs of its vertical-bar example (examples/Vertical_bar/*.data in
the Karamelo tree: the logs of a 3-D TLMPM, MUSL, FLIP 0.99, cubic-spline
neo-Hookean bar hanging under 1000 m/s^2, one line per step with columns
Step, dt, Time, fbody_x, fbody_y, fbody_z, dy_tip).  The first 121 lines of
five logs are kept: FLIP with the cubic spline at N = 10 (one particle per
cell) and N = 20 (two), FLIP with the linear basis at N = 20 (one), and APIC
with the cubic spline and with the linear basis at N = 20 (two).
Run where the Karamelo tree is available:

    python tests/golden/make_vertical_bar_golden.py path/to/Karamelo
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LOGS = {"n10_ppc1": "FLIP_99_cubic-spline_N-10_1_particle_per_cell.data",
        "n20_ppc2": "FLIP_99_cubic-spline_N-20_2_particle_per_cell.data",
        "linear_n20_ppc1": "FLIP_99_linear_N-20_1_particle_per_cell.data",
        "apic_n20_ppc2": "APIC_cubic-spline_N-20_2_particle_per_cell.data",
        "apic_linear_n20_ppc2": "APIC_linear_N-20_2_particle_per_cell.data"}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_vertical_bar_golden.py <root of the Karamelo tree>")
    root = sys.argv[1]
    out = {}
    for key, name in LOGS.items():
        a = np.genfromtxt(os.path.join(root, "examples", "Vertical_bar", name), skip_header=1)[:121]
        assert np.array_equal(a[:, 0], np.arange(len(a))), name
        out[f"{key}_dt"] = a[:, 1]
        out[f"{key}_time"] = a[:, 2]
        out[f"{key}_fbody_y"] = a[:, 4]
        out[f"{key}_dy_tip"] = a[:, 6]
    np.savez_compressed(os.path.join(HERE, "vertical_bar_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "vertical_bar_golden.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
