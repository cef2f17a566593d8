"""Build recipe for the oracle restatement (oracle/pfast_oracle.cpp ->
oracle/liboracle.so).  Test infrastructure only.

-ffp-contract=off matters: GCC contracts a*b+c into FMA by default on aarch64,
which would change the bits; the reference's arithmetic has no FMA.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def build(verbose=False):
    src = os.path.join(HERE, "pfast_oracle.cpp")
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC", "-shared",
           "-Wall", src, "-o", LIB, "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
