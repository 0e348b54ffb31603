"""CPU oracle (test infrastructure only): a C++ restatement of the reference
MPM substep, loaded through ctypes.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs use it; the product never does."""

from .oracle import *  # noqa: F401,F403
