"""Extract golden exact-Riemann star states from the reference's test data.

Reads Tests/RiemannProblems/Test*/exact/RiemannSolution.txt (written by the
reference's solver with PRINT_RIEMANN_SOLUTION, ExactRiemannSolverBase.cpp:535-556)
and the materials of each Test*/input.st, and writes riemann_star_states.json
beside this script: left/right states and IDs from the file header, the EOS
parameters, and the star states (rho*_L, rho*_R, u*, p*) read at the contact
(the row with xi = u*, and the row before it at xi = u* - max(1e-6, 1e-3|u*|),
ExactRiemannSolverBase.cpp:366-368).  Test7 (JWL equation of state) is skipped.

Usage: python tests/golden/make_riemann_golden.py <reference_dir>   (or M2C_REFERENCE_DIR)
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("M2C_REFERENCE_DIR")
if not REF:
    sys.exit("usage: %s <reference_dir> (or set M2C_REFERENCE_DIR)" % sys.argv[0])
HERE = os.path.dirname(os.path.abspath(__file__))
# IoData defaults (IoData.cpp:708-722 for Mie-Gruneisen)
MG_DEFAULT = dict(rho0=8.96e-3, c0=3.933e6, Gamma0=1.99, s=1.5, e0=0.0)


def strip_comments(txt):
    return re.sub(r"//[^\n]*", "", txt)


def parse_materials(txt):
    txt = strip_comments(txt)
    mats = {}
    for m in re.finditer(r"Material\[(\d+)\]\s*\{", txt):
        idx = int(m.group(1))
        depth, i = 1, m.end()
        while depth and i < len(txt):
            depth += {"{": 1, "}": -1}.get(txt[i], 0)
            i += 1
        body = txt[m.end():i]

        def num(key, default=None):
            r = re.search(rf"\b{key}\s*=\s*([-+0-9.eE]+)\s*;", body)
            return float(r.group(1)) if r else default
        eos = re.search(r"EquationOfState\s*=\s*(\w+)", body).group(1)
        d = dict(pmin=num("PressureCutOff", None), rhomin=num("DensityCutOff", None))
        if eos == "StiffenedGas":
            d.update(eos="SG", gamma=num("SpecificHeatRatio", 1.4), pc=num("PressureConstant", 0.0))
        elif eos == "NobleAbelStiffenedGas":
            d.update(eos="NASG", gamma=num("SpecificHeatRatio", 1.4), pc=num("PressureConstant", 0.0),
                     b=num("VolumeConstant", 0.0), q=num("EnergyConstant", 0.0))
        elif eos == "MieGruneisen":
            d.update(eos="MG", rho0=num("ReferenceDensity", MG_DEFAULT["rho0"]),
                     c0=num("BulkSpeedOfSound", MG_DEFAULT["c0"]), s=num("HugoniotSlope", MG_DEFAULT["s"]),
                     Gamma0=num("ReferenceGamma", MG_DEFAULT["Gamma0"]),
                     e0=num("ReferenceSpecificInternalEnergy", MG_DEFAULT["e0"]))
        else:
            d.update(eos=eos)
        mats[idx] = d
    return mats


def parse_solution(path):
    rows, header = [], None
    for line in open(path):
        if line.startswith("## Initial State"):
            nums = [float(x) for x in re.findall(r"[-+]?\d\.\d+e[-+]\d+", line)]
            ids = [int(x) for x in re.findall(r"id (\d+)", line)]
            header = dict(left=nums[0:3], right=nums[3:6], idl=ids[0], idr=ids[1])
        elif line.startswith("#") or not line.strip():
            continue
        else:
            rows.append([float(x) for x in line.split()])
    return header, rows


def star_states(rows):
    for i, r in enumerate(rows):
        xi, rho, u, p = r[:4]
        if abs(xi - u) <= 2e-6 * max(abs(u), 1e-30) + 1e-300 and i > 0:
            l = rows[i - 1]
            return dict(u_star=u, p_star=p, rho_l_star=l[1], rho_r_star=rho)
    return None


def main():
    out = []
    base = os.path.join(REF, "Tests", "RiemannProblems")
    for t in range(1, 13):
        d = os.path.join(base, f"Test{t}")
        sol = os.path.join(d, "exact", "RiemannSolution.txt")
        if not os.path.exists(sol):
            continue
        mats = parse_materials(open(os.path.join(d, "input.st")).read())
        if any(m["eos"] not in ("SG", "NASG", "MG") for m in mats.values()):
            continue
        header, rows = parse_solution(sol)
        st = star_states(rows)
        if st is None:
            continue
        out.append(dict(test=f"Test{t}", materials=[mats[k] for k in sorted(mats)], **header, **st,
                        source=f"Tests/RiemannProblems/Test{t}/exact/RiemannSolution.txt"))
    path = os.path.join(HERE, "riemann_star_states.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out)} cases to {path}")


if __name__ == "__main__":
    main()
