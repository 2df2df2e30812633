"""TEST INFRASTRUCTURE: the CPU oracle for the FFTCC -> IC-GN1 path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this package, and
only as the checker or the timed CPU baseline.  The product (fasticgn_gb300) never does.
"""
