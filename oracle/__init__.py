"""CPU oracle for the NRAPS Monte Carlo path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this package.  The product (nraps_gb300) never does.
"""
