"""Builds the oracle (oracle.cpp, scenes.cpp -> _build/liboracle.so) and, where the reference sources are
present, the reference harness (build_ref.sh -> _ref/libref_bbvh.so).

Test infrastructure: called by __graft_entry__.build() and by the tests; nothing in the
product links or loads these libraries.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where this recipe looks for the reference checkout unless GRT_REFERENCE_DIR names another
REFERENCE_CHECKOUT = "/root/reference"


def build(with_reference: bool = True) -> None:
    out = os.path.join(HERE, "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "scenes.cpp")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(s) for s in srcs):
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-o", so] + srcs, check=True)
    if with_reference:
        env = dict(os.environ)
        env.setdefault("GRT_REFERENCE_DIR", REFERENCE_CHECKOUT)
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True, stdout=subprocess.DEVNULL, env=env)


if __name__ == "__main__":
    build(with_reference="--no-ref" not in sys.argv)
    print("oracle built")
