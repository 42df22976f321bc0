"""ctypes binding of libdiffrp_gb300.so (the C ABI in include/diffrp_gb300.h).

The library is loaded from ``diffrp_gb300/_lib`` (built in-tree by
``diffrp_gb300.build``).  There is no CPU fallback: if the library is missing
or fails to load, every entry point raises.
"""
import ctypes
import os
import threading

_P = ctypes.c_void_p
_LL = ctypes.c_longlong
_ULL = ctypes.c_ulonglong
_I = ctypes.c_int
_F = ctypes.c_float
_SZ = ctypes.POINTER(ctypes.c_size_t)

_SIGNATURES = {
    "drp_abi_version": [],
    "drp_raster_workspace_size": [_I, _LL, _I, _I, _I, _ULL, _SZ],
    "drp_rasterize_fwd": [_P, ctypes.c_size_t, _P, _LL, _LL, _P, _LL, _I, _P, _LL, _I, _I, _I, _I, _ULL,
                          ctypes.c_uint, _P, _P, _P, _P, _P],
    "drp_rasterize_bwd": [_P, _LL, _LL, _P, _LL, _I, _I, _I, _P, _P, _P, _P, _P],
    "drp_interpolate_fwd": [_P, _LL, _LL, _I, _P, _P, _P, _LL, _I, _I, _I, _P, _I, _P, _P, _P],
    "drp_interpolate_bwd": [_P, _LL, _LL, _I, _P, _P, _P, _LL, _I, _I, _I, _P, _I, _P, _P, _P, _P, _P, _P],
    "drp_interpolate_sparse_fwd": [_P, _LL, _I, _P, _P, _LL, _P, _P],
    "drp_interpolate_sparse_bwd": [_P, _LL, _I, _P, _P, _LL, _P, _P, _P, _P],
    "drp_topology_workspace_size": [_LL, _SZ],
    "drp_antialias_topology": [_P, ctypes.c_size_t, _P, _LL, _P, _P],
    "drp_antialias_workspace_size": [_I, _LL, _SZ],
    "drp_edge_gradient_bwd": [_P, _P, _LL, _P, _P, _I, _P, _I, _I, _P, _P],
    "drp_l1_loss_workspace_size": [_LL, _SZ],
    "drp_l1_loss_fwd": [_P, ctypes.c_size_t, _P, _P, _LL, _F, _P, _P, _P],
    "drp_transform_points_fwd": [_P, _LL, _P, ctypes.c_int, _P, _P],
    "drp_transform_points_bwd": [_P, _LL, _P, ctypes.c_int, _P, _P],
    "drp_host_device_pointer": [_P, _P],
    "drp_copy_async": [_P, _P, ctypes.c_size_t, _P],
    "drp_antialias_fwd_noalloc": [_P, _I, _P, _P, _LL, _LL, _P, _LL, _P, _I, _I, _I, _P, _P],
    "drp_antialias_state_size": [_I, _I, _I, _SZ],
    "drp_antialias_fwd": [_P, ctypes.c_size_t, _P, _I, _P, _P, _LL, _LL, _P, _LL, _P, _I, _I, _I, _P, _P, _P],
    "drp_antialias_bwd": [_P, ctypes.c_size_t, _P, _I, _P, _P, _LL, _LL, _P, _LL, _P, _I, _I, _I, _P, _F, _P, _P,
                          _P, _P],
    "drp_texture_levels": [_I, _I, _I, ctypes.POINTER(ctypes.c_int)],
    "drp_texture_pyramid_floats": [_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_longlong)],
    "drp_texture_mip_build": [_P, _I, _I, _I, _I, _I, _P, _P],
    "drp_texture_fwd": [_P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P],
    "drp_texture_bwd": [_P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P],
}

ABI_VERSION = 1

_lib = None
_lock = threading.Lock()


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libdiffrp_gb300.so")


def load():
    """Load (once) and return the CUDA library; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    "diffrp_gb300 CUDA library not built (%s missing); run `python -m diffrp_gb300.build`" % path)
            lib = ctypes.CDLL(path)
            for name, argtypes in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = argtypes
                fn.restype = ctypes.c_int
            lib.drp_status_string.restype = ctypes.c_char_p
            lib.drp_status_string.argtypes = [ctypes.c_int]
            lib.drp_last_error.restype = ctypes.c_char_p
            lib.drp_last_error.argtypes = []
            lib.drp_kernel_launches.restype = ctypes.c_ulonglong
            lib.drp_kernel_launches.argtypes = []
            if lib.drp_abi_version() != ABI_VERSION:
                raise RuntimeError("libdiffrp_gb300 ABI %d != expected %d" % (lib.drp_abi_version(), ABI_VERSION))
            _lib = lib
    return _lib


_fast = None


def _fast_table():
    """Entry points of the CPython fast path (csrc/pyext.cpp), or {} when it
    was not built; the library itself must already be loaded."""
    global _fast
    if _fast is None:
        table = {}
        path = os.path.join(os.path.dirname(lib_path()), "_drp_fast.so")
        if os.path.exists(path) and not os.environ.get("DRP_NO_FAST_PATH"):
            import importlib.machinery
            import importlib.util
            try:
                loader = importlib.machinery.ExtensionFileLoader("_drp_fast", path)
                spec = importlib.util.spec_from_file_location("_drp_fast", path, loader=loader)
                mod = importlib.util.module_from_spec(spec)
                loader.exec_module(mod)
                table = {k: getattr(mod, k) for k in dir(mod) if k.startswith("drp_")}
            except ImportError:
                table = {}
        _fast = table
    return _fast


def call(name, *args):
    """Call an entry point; a non-zero status becomes RuntimeError."""
    lib = load()
    fn = (_fast if _fast is not None else _fast_table()).get(name)
    status = fn(*args) if fn is not None else getattr(lib, name)(*args)
    if status != 0:
        msg = lib.drp_last_error().decode(errors="replace")
        raise RuntimeError("%s failed (%s): %s" % (name, lib.drp_status_string(status).decode(), msg))
    return status


_sizes = {}


def size_out(name, *args):
    """A workspace-size query (a pure function of its integer arguments),
    answered from a cache after the first call."""
    key = (name,) + args
    v = _sizes.get(key)
    if v is None:
        out = ctypes.c_size_t(0)
        call(name, *args, ctypes.byref(out))
        v = _sizes[key] = out.value
    return v


def stream_of(device):
    """Raw cudaStream_t (as an int) of the current torch stream on device."""
    import torch
    idx = device.index if device.index is not None else torch.cuda.current_device()
    return torch._C._cuda_getCurrentRawStream(idx)


def kernel_launches():
    """Kernel launches the library has enqueued so far (graph captures count
    each captured launch once)."""
    return int(load().drp_kernel_launches())
