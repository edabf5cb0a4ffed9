"""CPU oracle for the libKriging likelihood path: TEST AND BENCH-BASELINE INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use this package; the GPU
product never imports it.
"""
