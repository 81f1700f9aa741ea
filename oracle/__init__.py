"""ORACLE - test infrastructure only.

CPU restatement of the reference's time-stepping path: the oracle that the
CUDA path is compared with (tests, smoke check) and the timed CPU baseline of
the benchmark. The product package never imports it.
"""
