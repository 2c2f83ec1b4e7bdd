"""CPU oracle of the smoke step -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this package, and only to check results.  The product library
(zq_smokesimulation_gb300) never imports, links or calls it.
"""
