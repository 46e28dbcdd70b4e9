"""Oracle for the fv3d hydro step -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only for the results the GPU path is compared with / the
timed CPU baseline.  The product
(fv3d_gb300) never imports, links or executes anything here.
"""
