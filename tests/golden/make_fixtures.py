"""Writes the golden fixtures of tests/golden from the reference checkout.

Run once where the NREL/marbles sources are present, giving the path of the
checkout (required):
    python tests/golden/make_fixtures.py <path-to-marbles-checkout>
It reads, as text only:
  * Source/Stencil.H     -> stencil_d3q27.json: the D3Q27 direction table,
                            the four bounce tables and the weight expressions
  * Tools/viscosity_test/viscosity_tester.ipynb and
    Tools/thermaldiffusivity_test/thermaldiffusivity_tester.ipynb
                         -> notebook_runs.json: the recorded max-value time
                            series of the reference's own runs (every 5000
                            steps) with the inputs they were produced with.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def stencil(ref):
    src = open(os.path.join(ref, "Source", "Stencil.H")).read()
    body = src[src.index("#else"):]
    evs = re.findall(r"amrex::IntVect\(\s*([-\w]+)\s*,\s*([-\w]+)\s*,\s*([-\w]+)\s*\)", body)
    val = {"0": 0, "CSC1": 1, "-CSC1": -1, "CFCC1": 1, "-CFCC1": -1, "CBCC1": 1, "-CBCC1": -1}
    ev = [[val[a], val[b], val[c]] for a, b, c in evs]
    enum = re.search(r"enum dvD3Q27 \{(.*?)\};", body, re.S).group(1)
    names = [n.strip() for n in enum.replace("\n", " ").split(",") if n.strip()]
    idx = {n: i for i, n in enumerate(names)}
    tables = {}
    for t in ["bounce_dirs", "bounce_Xdir", "bounce_Ydir", "bounce_Zdir"]:
        m = re.search(t + r" = \{(.*?)\};", body, re.S).group(1)
        tables[t] = [idx[n.strip()] for n in m.replace("\n", " ").split(",") if n.strip()]
    return {"source": "Source/Stencil.H", "ev": ev, **tables,
            "weights": {"WSC1": "2/27", "WFCC1": "1/54", "WBCC1": "1/216",
                        "WO": "1 - (6*WSC1 + 12*WFCC1 + 8*WBCC1)"}}


def notebook_lists(path, name):
    nb = json.load(open(path))
    code = "".join(nb["cells"][1]["source"])
    out = []
    for line in code.splitlines():
        m = re.match(r"\s*#?\s*" + name + r"\s*=\s*\[(.*)\]", line)
        if m:
            out.append([float(v) for v in m.group(1).split(",") if v.strip()])
    return code, out


def notebooks(ref):
    vcode, vl = notebook_lists(os.path.join(ref, "Tools", "viscosity_test", "viscosity_tester.ipynb"), "uxMaxList")
    tcode, tl = notebook_lists(os.path.join(ref, "Tools", "thermaldiffusivity_test",
                                            "thermaldiffusivity_tester.ipynb"), "temperatureMaxList")
    # the uncommented list of each notebook is the one its header describes
    vsel = [l for l in vcode.splitlines() if l.startswith("uxMaxList")][0]
    tsel = [l for l in tcode.splitlines() if l.startswith("temperatureMaxList")][0]
    vsel = [float(v) for v in vsel.split("[")[1].split("]")[0].split(",")]
    tsel = [float(v) for v in tsel.split("[")[1].split("]")[0].split(",")]
    return {
        "viscosity_test": {
            "source": "Tools/viscosity_test/viscosity_tester.ipynb cell 1 (uncommented list), "
                      "Tests/test_files/viscosity_test/viscosity_test.inp",
            "inputs": {"n_cell": [6, 200, 2], "prob_lo": [0.0, 0.0, -1.0], "prob_hi": [6.0, 200.0, 1.0],
                       "nu": 1e-4, "initial_temperature": 0.3333, "adiabatic_exponent": 5.0 / 3.0,
                       "mean_molecular_mass": 28.96, "wave_length": 200.0},
            "interval": 5000, "ux_max": vsel},
        "thermaldiffusivity_test": {
            "source": "Tools/thermaldiffusivity_test/thermaldiffusivity_tester.ipynb cell 1 (uncommented list), "
                      "Tests/test_files/thermaldiffusivity_test/thermaldiffusivity_test.inp",
            "inputs": {"n_cell": [6, 200, 2], "prob_lo": [0.0, 0.0, -1.0], "prob_hi": [6.0, 200.0, 1.0],
                       "nu": 8.76e-6, "alpha": 1e-5, "initial_temperature": 0.003333,
                       "adiabatic_exponent": 1.32, "mean_molecular_mass": 17.031, "wave_length": 200.0},
            "interval": 5000, "t_max": tsel},
    }


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <path-to-marbles-checkout>")
    ref = sys.argv[1]
    json.dump(stencil(ref), open(os.path.join(HERE, "stencil_d3q27.json"), "w"), indent=1)
    json.dump(notebooks(ref), open(os.path.join(HERE, "notebook_runs.json"), "w"), indent=1)
    print("wrote fixtures to", HERE)
