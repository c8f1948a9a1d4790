"""FP64 CPU restatement of the reference MPM step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product (libaep.so) never
uses it.  Parity unpinned: the reference cannot be built here and ships no
golden vectors; see aep_oracle.cpp.
"""
