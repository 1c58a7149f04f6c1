"""vectra_gb300: GB300 (sm_103a) operator nodes for vectra's columnar
execution path, behind the reference's own node C API (include/vgpu.h).

`load()` opens the in-tree libvgpu.so; it raises if the library has not been
built -- there is no CPU fallback.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvgpu.so")

_lib = None


def load():
    """The libvgpu shared library (ctypes.CDLL)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libvgpu.so is not built: run `python -m vectra_gb300.build` "
                               "(or __graft_entry__.build())")
        _lib = C.CDLL(LIB_PATH)
        _lib.vgpu_init.restype = C.c_int
        _lib.vgpu_init.argtypes = [C.c_int]
        _lib.vgpu_last_error.restype = C.c_char_p
        _lib.vgpu_kernel_launches.restype = C.c_ulonglong
        _lib.vgpu_set_stream.argtypes = [C.c_void_p]
        _lib.vgpu_get_stream.restype = C.c_void_p
        _lib.vgpu_synchronize.restype = C.c_int
        _lib.vgpu_warning_count.restype = C.c_long
    return _lib


def engine(device=0):
    """A plan engine bound to libvgpu on `device` (initialises CUDA)."""
    from .plan import GpuEngine
    lib = load()
    if lib.vgpu_init(device) != 0:
        raise RuntimeError("libvgpu: " + lib.vgpu_last_error().decode())
    return GpuEngine(lib)
