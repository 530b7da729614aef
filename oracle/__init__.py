"""Test infrastructure: the oracle (CPU restatement of the reference hot path)
and the recipe that compiles the reference itself where its sources exist.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it."""
