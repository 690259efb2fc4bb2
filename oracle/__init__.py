"""CPU oracle for the euc triangle pipeline (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this package.  PARITY UNPINNED: euc ships no golden outputs and cannot run
here; see euc_oracle.cpp's header.
"""
