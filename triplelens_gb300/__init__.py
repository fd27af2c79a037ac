"""GB300-native engine for TripleLens' extended-source light curves.

The product is the shared library ``bin/liblcirs.so`` (C ABI in
``include/lcirs.h``), a drop-in for the reference's ``liblcirs.so``.  This
package holds its CUDA sources (``csrc/``), the build recipe and a ctypes
mirror of the reference's Python classes (``LC_irs``, ``CCC``).
"""
from .lcirs import LC_irs, load_lcirs  # noqa: F401
