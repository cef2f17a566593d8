"""CPU oracle for PFAST's traveltime + adjoint-state path (test infrastructure).

`oracle.port` wraps the restatement in pfast_oracle.cpp; `oracle.ref` wraps the
reference's own headers built into oracle/_ref (present only where the
reference tree was available at build time).  Only tests/, the smoke check and
bench.py's CPU baseline legs use this package; the CUDA library never does.
"""
