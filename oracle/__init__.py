"""CPU oracle of the wavefront path tracer — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
this.  See oracle.h for what it restates and its parity status.
"""
