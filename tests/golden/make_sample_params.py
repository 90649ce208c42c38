"""Extracts the key/value lines of the reference's eight sample parameter
files (param.txt, paramSphere.txt, paramPear.txt, input_parameters.txt,
test1.txt .. test4.txt at the root of the McLiCS tree) into
reference_samples.json: comments and blank lines dropped, keys and values as
written.  tests/test_abi.py runs every one through mcx_check_file.

    python tests/golden/make_sample_params.py <McLiCS source tree>
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ["param.txt", "paramSphere.txt", "paramPear.txt", "input_parameters.txt", "test1.txt", "test2.txt",
         "test3.txt", "test4.txt"]


def main():
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    out = {}
    for name in FILES:
        lines = []
        with open(os.path.join(sys.argv[1], name), encoding="utf-8", errors="replace") as f:
            for ln in f:
                body = ln.split("#", 1)[0].strip()
                if body:
                    lines.append(" ".join(body.split()))
        out[name] = "\n".join(lines) + "\n"
    with open(os.path.join(HERE, "reference_samples.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out)} sample parameter files")


if __name__ == "__main__":
    main()
