"""Oracle for the convolution library — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package, and only to check or time against it; the product
(``arrayfire_gb300``) never does.
"""
from .oracle import *  # noqa: F401,F403
