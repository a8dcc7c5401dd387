"""CPU restatement of the kazen_proto hot path — test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg as the
checker / reference timing; never by the product package.
"""
