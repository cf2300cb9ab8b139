"""Regenerate tests/golden/reference_golden.json from the reference itself.

Builds the reference library from its sources (oracle/ref_build.sh, outputs in
oracle/_ref/) and runs oracle/ref_recorder.cpp, which drives the reference
through its public API.  Needs the reference checkout, given as the argument or in
the environment variable MCIG_REFERENCE_ROOT; the committed JSON is what the tests
read, so nothing at test time needs it.

    python tests/golden/make_golden.py REFERENCE_ROOT
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCIG_REFERENCE_ROOT", "")
    if not ref:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set MCIG_REFERENCE_ROOT)")
    subprocess.check_call([os.path.join(ROOT, "oracle", "ref_build.sh"), ref])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_recorder")])
    data = json.loads(out)  # validate
    with open(os.path.join(HERE, "reference_golden.json"), "wb") as f:
        f.write(out)
    print("wrote %d entries" % len(data))


if __name__ == "__main__":
    main()
