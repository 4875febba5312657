"""Builds the CPU oracle (oracle/pdhg_oracle.cpp) into oracle/_build/libpdhg_oracle.so.

The oracle is test infrastructure: tests/, __graft_entry__.smoke() and bench.py's CPU
legs load it; the product never does. Plain g++ with OpenMP, no FMA contraction, so
its arithmetic follows the reference's operation order.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpdhg_oracle.so")
# The same oracle with another summation order (64-element reduction chunks, rows of
# every product summed last-to-first). The reference loop is chaotic in floating point,
# so the distance between the two oracles measures how far two correct implementations
# that only round differently drift apart; GPU parity is checked against that envelope.
LIB_PERTURBED = os.path.join(OUT_DIR, "libpdhg_oracle_perturbed.so")
SRC = os.path.join(HERE, "pdhg_oracle.cpp")


def _build_one(out, defines, force):
    hdr = os.path.join(HERE, "..", "include", "gpdhg.h")
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", *defines,
           SRC, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    _build_one(LIB_PERTURBED, ["-DORACLE_CHUNK=64", "-DORACLE_REVERSE_SPMV"], force)
    return _build_one(LIB, [], force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
