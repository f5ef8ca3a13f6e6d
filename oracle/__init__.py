"""Oracles for DiaQ's diagonal-sparse hot path -- TEST INFRASTRUCTURE ONLY.

``oracle.oracle``    the C restatement (diaq_oracle.c) and the host algorithms over it.
``oracle.reference`` the reference's own CPU code, where it was built (oracle/_ref/).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference leg may import
this package; the product path never does.
"""
