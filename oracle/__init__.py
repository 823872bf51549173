"""Test infrastructure: the FP64 CPU oracle and the reference harness.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package. The product (the CUDA library) never imports it.
"""
