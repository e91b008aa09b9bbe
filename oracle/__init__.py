"""CPU oracle for the cuYASHE hot path.

This package is test infrastructure. Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg (and its ``--impl reference`` arm) may import
it, and only to check or to time against. The GPU product never calls it.

Contents
--------
ring      exact arithmetic in Z_q[x]/(x^N+1) with Python integers: schoolbook and
          Kronecker-substitution negacyclic products, the reference's ``reduce``
          (fold by x^N+1, then mod q), CRT/ICRT round trips.
yashe     the YASHE scheme of Bos, Lauter, Loftus and Naehrig (2013) as the
          reference intends it (``src/yashe.cpp``, ``src/ciphertext.cpp``), with
          the defects listed in its docstring corrected: a real f^-1, the t/q
          rounding over Z, base-2^w word decomposition and full-polynomial
          decryption.
refpath   ctypes wrapper around ``refpath.c``: a C restatement of the reference's
          own multiply (29-bit CRT bucket, Goldilocks radix-2 Stockham NTT,
          integer NTTScale, ICRT, fold + mod q). It is the timed CPU baseline and
          the parity target where the reference is correct (N <= 8).
"""
