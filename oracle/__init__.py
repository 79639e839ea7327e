"""CPU oracle of the pyCudaPolygon hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline legs may
import this package.  The CUDA product path never calls it.
"""
