"""CPU oracle of the LucidRaster compute raster path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this package; the
lucid_gb300 product path never imports it.
"""
