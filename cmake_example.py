"""Top-level ``cmake_example``: the module name the reference's Python driver imports.

FastPGM's python/pyfastpgm.py starts with ``import cmake_example as fastpgm`` (the pybind11
module of python/api_main.cpp:9-12).  With this repository on PYTHONPATH that line imports
this module, which re-exports the GB300 engine's drop-in functions with the reference's
names and positional arguments, so pyfastpgm.py runs unchanged.
"""
import os
import sys

_ROOT = os.path.dirname(os.path.abspath(__file__))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from fastpgm_gb300.cmake_example import BNL_PCStable, BNSL_PCStable  # noqa: E402,F401

__all__ = ["BNSL_PCStable", "BNL_PCStable"]
