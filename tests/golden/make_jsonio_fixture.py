"""Copy the reference's JSON-index fixture (utils/iocore/jsonio_expected.json, the expected
output of utils/iocore/jsonio_test.f90) to tests/golden/jsonio_expected.json.  It pins the
json-fortran text format that the restart writer reproduces.

Run from the repository root, giving the path of a WumingPIC checkout:
    python tests/golden/make_jsonio_fixture.py <path-to-WumingPIC>
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_jsonio_fixture.py <path-to-WumingPIC>")
    ref = sys.argv[1]
    shutil.copyfile(os.path.join(ref, "utils", "iocore", "jsonio_expected.json"),
                    os.path.join(HERE, "jsonio_expected.json"))
