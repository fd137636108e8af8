"""Golden end-of-run line plots of the reference's own tests.

For every Tests/RiemannProblems/Test*/ directory of the reference (Test7, JWL,
skipped) and the two-dimensional Tests/ExplosionShyue98 case: the input file
parsed by m2c_gb300.inputfile.parse (the nested
key/value tree, which the tests turn into a configuration and initial state
with Case.from_tree), and the final line plot results/line_0001.txt written
by the reference (ProbeOutput.cpp:483-597): time, time step and the columns
density, velocity x, pressure, material ID and level set at the line's points.
Writes reference_lines.json beside this script.

Usage: python tests/golden/make_reference_lines.py <reference_dir>   (or M2C_REFERENCE_DIR)
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from m2c_gb300.inputfile import parse  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("M2C_REFERENCE_DIR")
if not REF:
    sys.exit("usage: %s <reference_dir> (or set M2C_REFERENCE_DIR)" % sys.argv[0])


def main():
    base = os.path.join(REF, "Tests", "RiemannProblems")
    dirs = [(name, os.path.join(base, name)) for name in sorted(os.listdir(base), key=lambda s: (len(s), s))
            if name.startswith("Test") and name != "Test7"]
    dirs.append(("ExplosionShyue98", os.path.join(REF, "Tests", "ExplosionShyue98")))
    out = {}
    for name, d in dirs:
        tree = parse(open(os.path.join(d, "input.st")).read())
        lines = open(os.path.join(d, "results", "line_0001.txt")).read().splitlines()
        m = re.match(r"## Time: (\S+), Time step: (\d+)\.", lines[2])
        rows = [[float(v) for v in ln.split()] for ln in lines if ln and not ln.startswith("#")]
        cols = list(zip(*rows))
        out[name] = {"tree": tree, "time": float(m.group(1)), "step": int(m.group(2)),
                     "rho": cols[1], "vx": cols[2], "p": cols[5], "id": cols[7],
                     "phi": cols[8] if len(cols) > 8 else None}
    with open(os.path.join(HERE, "reference_lines.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
