"""Test infrastructure (the oracle).  Imported only by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, to check results against.  The product package never imports it."""
