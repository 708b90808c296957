"""The checker for the render path: TEST INFRASTRUCTURE ONLY.

oracle.oracle  -- CPU restatement of the reference's algorithm (C, ctypes)
oracle.ref     -- driver for the reference's own kernels (built from its sources)
oracle.build   -- build recipe for both

Only tests/, __graft_entry__.smoke() and bench.py's baseline legs use this
package; jaxsplat_gb300 never imports it.
"""
