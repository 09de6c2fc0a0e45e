"""Oracle for t1m_gb300 — TEST INFRASTRUCTURE, not product code.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker (or the timed
CPU baseline).  The product library never links or calls it.

* ``numpy_oracle`` — numpy restatement of the reference's index bundling,
  scatter/block-scatter, 1M packing/unpacking (include/t1m/t1m.h) and the
  FP64 einsum oracle.
* ``port/t1m_port.cpp`` — C++ restatement of the full five-loop 1M algorithm,
  bit-identical to the reference built against the same BLIS stand-in.
* ``ref_shim.cpp`` — instantiates the unmodified reference headers (built only
  where the reference tree exists, into ``oracle/_ref/``).

Parity pin: BLIS itself is absent (third-party, unpinned), so the exact bits of
the reference's BLIS micro-kernel are unpinned; the stand-in micro-kernel in
``standin/blis.h`` replaces it on both the reference and the port.
"""
