"""CPU oracle of the EasyFEA hot path -- TEST INFRASTRUCTURE ONLY.

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``, as the checker.  The product package never imports it.
Parity pinned against fixtures generated from the reference itself
(``tests/golden/make_golden.py``).
"""
