"""CPU oracle of the KPM moment path: test infrastructure, never the product.

Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline may use this package.
"""
