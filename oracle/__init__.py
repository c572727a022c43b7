"""Test infrastructure only: the CPU restatement (oracle) of Tina's raster +
shade path.  Imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg -- never by the taichi_three_gb300 package."""
