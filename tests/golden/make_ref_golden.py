"""Golden fixtures from the reference itself.

Builds the reference (every src/*.cpp of the Karamelo tree, unmodified,
against oracle/stubs) and its full-precision driver oracle/_ref/ref_harness,
runs each case of tests/golden/ref_cases.py through it, and writes
tests/golden/ref_<case>.npz.

    python tests/golden/make_ref_golden.py --karamelo <Karamelo tree> [case ...]

The tree is a required argument; the fixtures are committed, so the tests
need neither the tree nor the harness.
"""
import argparse
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import ref_cases as RC  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--karamelo", required=True, help="root of the Karamelo source tree")
    ap.add_argument("cases", nargs="*", help="cases to make (default: all)")
    a = ap.parse_args()
    src = os.path.join(os.path.abspath(a.karamelo), "src")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_SRC={src}", "-j8"])
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    for name in a.cases or list(RC.CASES):
        script = RC.reference_script(name)
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "case.mpm"), "w") as f:
                f.write(script)
            t0 = time.time()
            r = subprocess.run([harness, "case.mpm", "out.bin"], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                sys.exit(f"{name}: reference run failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            recs = RC.read_harness(os.path.join(d, "out.bin"))
        arrays = RC.pack(recs)
        out = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(out, **arrays)
        print(f"{name}: {len(recs)} records, {time.time() - t0:.1f} s, {os.path.getsize(out) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
