"""GB300-native short-range pair-force engine for AutoPas (LJ 12-6, Verlet cluster lists, velocity Verlet).

The compute path is hand-written CUDA for sm_103a in ``csrc/``, built into ``lib/libpairengine.so`` with the
C ABI of ``include/pairengine.h`` (``autopas_gb300.build.build()``).  ``engine.PairEngine`` is a ctypes
wrapper over that ABI; the C++ mirror of the AutoPas container / traversal / functor interface is in
``include/autopas_gb300/``.
"""
