"""TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference PRIME20
DMD engine (dmd_oracle.cpp) and its ctypes binding.  Imported only by
tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg."""
