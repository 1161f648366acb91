"""Extract the golden epsilon logs from the reference's recorded runs.

The reference project ships the epsilon-per-iteration logs of its line-search
drivers (data_dynamic/sirt-dyn-<gs>-<noise>.txt from sirt-test-weight.cu and
data_dynamic/sirt-norm-dyn-<gs>-<noise>.txt from sirt-norm-test-weight.cu).
Columns: iteration (1-based), epsilon %, epsilon decrease, best step size.
This script keeps the first rows of the noise-free logs as a fixture; the
tests replay each log's recorded step sizes in the oracle and compare epsilon.

Usage: python tests/golden/make_ref_logs.py /path/to/reference
"""
import json
import os
import sys

ROWS = 6


def main(ref_root: str) -> None:
    out = {}
    d = os.path.join(ref_root, "data_dynamic")
    for kind, method in (("sirt", "scaled"), ("sirt-norm", "norm")):
        for gs in (10, 20, 32, 160):
            name = f"{kind}-dyn-{gs}-0.txt"
            rows = []
            with open(os.path.join(d, name)) as fh:
                for line in fh:
                    parts = line.split()
                    if len(parts) == 4:
                        rows.append([int(parts[0]), float(parts[1]), float(parts[2]), float(parts[3])])
                    if len(rows) == ROWS:
                        break
            out[name] = {"group_size": gs, "method": method, "rows": rows}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_eps_logs.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_ref_logs.py <reference checkout>")
    main(sys.argv[1])
