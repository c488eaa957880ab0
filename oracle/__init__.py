"""CPU restatement of vserdyuk/cuda_als's ALS sweep: the checker.  TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs, never
by the cuda_als_gb300 package.
"""
