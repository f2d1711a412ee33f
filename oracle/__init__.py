"""Oracle (test infrastructure): CPU restatement of the reference's hot path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package: to check the GPU results, or as the timed CPU reference.  The GPU
product path never imports it.
"""
