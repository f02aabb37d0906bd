"""CPU oracle for the MARS forward pass (test infrastructure).

Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs
import this package. It is the checker and the CPU baseline, never the product:
``mars_gb300`` does not import it and has no CPU fallback.

* ``port``       -- ``oracle/mars_oracle.c``, a plain-C restatement of the
                    reference CPU path (built by ``oracle/Makefile``).
* ``ref``        -- the reference's own ``marsalgo.cc``/``kernels.cc`` compiled
                    where they lie (only where the reference sources exist).
* ``ref_scalar`` -- the same sources with the AVX branches compiled out; the
                    port must match it bit for bit.
"""
from .oracle import (  # noqa: F401
    OracleAlgo,
    OracleLib,
    build,
    load,
    marslib_for,
    available,
)
