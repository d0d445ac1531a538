"""CPU oracle for the FacetRT path — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this package.  The product library never calls it.
"""
