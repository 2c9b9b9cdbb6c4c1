"""CPU oracle for the BMND direct-Poisson path (test infrastructure only).

``oracle/bmnd_oracle.c`` restates the reference algorithm in C; this package
loads it from ``oracle/_ref/libbmnd_oracle.so`` (built by ``oracle/Makefile``)
and offers NumPy-level wrappers.  Only tests, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` use it, as the checker.
"""

from .oracle import *  # noqa: F401,F403
