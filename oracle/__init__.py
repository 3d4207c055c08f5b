"""ORACLE — test infrastructure only: a CPU restatement of the reference's trace path, used as the checker
by tests/ and the smoke check, and as the CPU baseline of bench.py.  Never imported by the product."""
