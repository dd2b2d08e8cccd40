"""Regenerates tests/golden/ref_vectors.json from the reference's own code.

Builds oracle/_ref/ref_harness (oracle/Makefile target `ref`), which compiles
the reference's FIRGaussianConvolver.cu together with its unmodified
FIRGaussianConvolver.h, GuidedFilter.h and Testprog/filterTest/filterImageGold.h
against small stand-ins for the TULibs headers, runs it, and stores its JSON
output.  Needs a reference checkout, named by $TUCU_REF or the first
argument; the committed fixture is what the tests read.

    TUCU_REF=<reference checkout> python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main() -> int:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TUCU_REF", "")
    if not ref or not os.path.isdir(ref):
        print(f"reference checkout not found at {ref}", file=sys.stderr)
        return 1
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}"],
                   check=True)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_harness")],
                         check=True, capture_output=True, text=True).stdout
    data = json.loads(out)
    data["_generated_by"] = "tests/golden/make_golden.py (oracle/ref_harness.cpp)"
    with open(os.path.join(HERE, "ref_vectors.json"), "w") as f:
        json.dump(data, f, separators=(",", ":"))
        f.write("\n")
    print("wrote", os.path.join(HERE, "ref_vectors.json"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
