"""ORACLE - test infrastructure only.

CPU restatement of the reference's time-stepping path, used as the checker of
the CUDA path (tests, smoke check) and as the timed CPU baseline of the
benchmark. The product package never imports it.
"""
