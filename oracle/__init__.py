"""CPU oracle of the MPS trajectory path (test infrastructure only: imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
product path)."""
