"""CPU oracle for the TUCuda 2D-filter path -- test infrastructure only.

Used by tests/, by __graft_entry__.smoke() as the checker and by bench.py's
CPU-baseline leg; the product path never imports it.
"""
