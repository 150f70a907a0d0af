"""Writes tests/golden/extrapolation_constants.json from the reference's unit-test outputs
(tests/time_integration/extrapolation_constants_0{1,2}.output: constant and adaptive time steps,
orders 1-4, each current order).  Run in a container that has the reference tree."""
import json
import os
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
out = {}
for name in ("extrapolation_constants_01", "extrapolation_constants_02"):
    path = os.path.join(REF, "tests", "time_integration", name + ".output")
    out[name] = open(path).read().splitlines()
json.dump(out, open(os.path.join(os.path.dirname(__file__), "extrapolation_constants.json"), "w"), indent=1)
