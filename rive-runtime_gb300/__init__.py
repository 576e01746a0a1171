"""GB300-native flush backend for the Rive vector renderer.

The product is the C-ABI shared library built from ``csrc/`` (declared in
``include/rive_cuda.h``). This package holds its Python-side helpers: the
ctypes binding (``rive_cuda``), the planner binding (``planner``), the seeded
scene generator (``scene``) and the flush-capture reader (``capture``).
"""
import os

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_ROOT = os.path.dirname(PACKAGE_DIR)
