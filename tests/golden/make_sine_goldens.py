"""Extract the reference's golden relative L2 errors of the sine application.

Reads applications/poisson/sine/tests/{cartesian,curvilinear}.output from the ExaDG source tree
(default /root/reference; first argument overrides) and writes sine_errors.json beside this file.
Each output file prints, per degree k = 1..7, the error of the initial data and then of the
solution; the second value per degree is the one kept.
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))


def read(name):
    path = os.path.join(ROOT, "applications", "poisson", "sine", "tests", name + ".output")
    txt = open(path).read()
    blocks = re.split(r"Calculate error for all fields for ", txt)
    sol = []
    for b in blocks[1:]:
        if b.startswith("solution data"):
            m = re.search(r"Relative error \(L2-norm\):\s*([0-9.eE+-]+)", b)
            sol.append(float(m.group(1)))
    degs = [int(x) for x in re.findall(r"Polynomial degree:\s*(\d+)", txt)]
    return {"degrees": degs, "relative_l2_error": sol, "source": "applications/poisson/sine/tests/%s.output" % name}


out = {
    "problem": {
        "domain": [-1.0, 1.0], "n_cells_1d": 8, "mapping_degree": 3, "ip_factor": 1.0,
        "solution": "prod_d sin(3 pi x_d)", "rhs": "27 pi^2 u", "dirichlet_sides": "all but x=+1",
        "neumann_side": "x=+1 (du/dx)", "curvilinear": {"deformation": 0.15, "frequency": 2},
        "solver": "CG rel 1e-10, abs 1e-20",
    },
    "cartesian": read("cartesian"),
    "curvilinear": read("curvilinear"),
}
with open(os.path.join(HERE, "sine_errors.json"), "w") as f:
    json.dump(out, f, indent=1)
print(json.dumps(out, indent=1))
