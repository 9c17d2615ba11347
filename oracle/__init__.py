"""The oracle: CPU restatement of the reference path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
import this package; the product (coldcase_gb300/) never does.
"""
