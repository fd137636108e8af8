"""Oracle: CPU restatement of the reference's hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as
the checker.  The product library never loads it."""
