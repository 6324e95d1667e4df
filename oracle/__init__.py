"""Test infrastructure: the CPU oracle (afar_oracle.c) and the reference-kernel harness
(ref_harness.cpp + cubins built from the reference sources).  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg import this package; the product path never does."""
