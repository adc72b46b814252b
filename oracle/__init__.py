"""ORACLE - test infrastructure only (see oracle/oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only to check results; the GPU library never uses it.
"""
