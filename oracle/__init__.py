"""TEST INFRASTRUCTURE: the CPU oracle for PhyloAcc-ST's per-element MCMC.

Used only by tests/, __graft_entry__.smoke() (as the checker) and bench.py's
CPU-baseline leg.  Nothing in the product imports it."""
