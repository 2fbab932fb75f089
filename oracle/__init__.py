"""CPU oracle of the renderer's path-tracing hot path (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package; the product path never does.
"""
