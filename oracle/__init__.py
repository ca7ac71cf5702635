"""CPU oracle for the cuJSON parse path -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker (and the timed CPU baseline).  The product never imports
it.  See cj_oracle.h for the contract and the reference lines it restates.
"""
