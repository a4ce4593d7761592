"""Parity oracle for the FWI hot path: a C restatement of the reference's CPU
algorithm (fwi_oracle.c) and the reference's own CPU path compiled from its
sources (build.py -> _ref/).  Test infrastructure only; the product
(cuda_fwi_gb300) never imports this package."""
