"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the Lomb-Scargle path.

A restatement of the reference's CPU algorithm (oracle/ls_oracle.c) and, when the
reference checkout is present, the recipe that builds the reference's own CPU
path into oracle/_ref/ (oracle/Makefile). Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline legs may use it; the product never does.
"""
