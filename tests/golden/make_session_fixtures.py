"""Writes tests/golden/session_helmholtz2d_p7_periodic.json: the reference session file
library/Demos/MultiRegions/Tests/Helmholtz2D_P7_Periodic.xml read by the library's
session reader (ithaca_gpu.session) and stored as plain data, so that the GPU tests,
which run without the reference tree, solve the same case.

Run where the reference tree is present:
    python tests/golden/make_session_fixtures.py [reference root]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.session import read_session  # noqa: E402

CASES = {"session_helmholtz2d_p7_periodic.json": "library/Demos/MultiRegions/Tests/Helmholtz2D_P7_Periodic.xml"}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ITHACA_REFERENCE", "/root/reference")
    for out, rel in CASES.items():
        s = read_session(os.path.join(ref, rel))
        with open(os.path.join(HERE, out), "w") as f:
            json.dump(dict(source=rel, session=s.to_dict()), f, indent=1, sort_keys=True)
        print("wrote", out)


if __name__ == "__main__":
    main()
