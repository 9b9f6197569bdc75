"""In-tree build of libsffg.so (nvcc for sm_103a + g++ host code)."""
import os

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")


def library_path():
    return os.environ.get("SFFG_LIBRARY", os.path.join(OUT, "libsffg.so"))
