"""Locations of the in-tree native libraries built by ``pargo_gb300.build``."""
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")
GPU_SO = os.path.join(LIB_DIR, "libpargo_gpu.so")
SYNTH_SO = os.path.join(LIB_DIR, "libpargo_synth.so")
GPRO_SO = os.path.join(LIB_DIR, "libpargo_gpro.so")
BIN_DIR = os.path.join(LIB_DIR, "bin")


class NativeLibraryMissing(ImportError):
    pass


def require(path):
    if not os.path.exists(path):
        raise NativeLibraryMissing(
            "%s is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(or `python -m pargo_gb300.build`) first" % path)
    return path
