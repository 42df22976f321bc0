// pyext.cpp -- a CPython fast path onto the C ABI of libdiffrp_gb300.so.
//
// ctypes spends several microseconds converting each call's arguments; the
// drop-in ops make a handful of calls per step, which adds up in eager
// PyTorch.  Each wrapper here takes the same positional arguments as the
// C function it names (device pointers and sizes as Python ints, None for
// NULL, floats as Python floats or ctypes.c_float) and returns the int
// status, so diffrp_gb300._ffi.call can use either path.  The argument
// unpacking is generated from the declarations in include/diffrp_gb300.h by
// the template below, so a wrapper cannot disagree with its function's types.
#define PY_SSIZE_T_CLEAN
#include <Python.h>

#include <cstddef>
#include <cstdint>
#include <tuple>
#include <type_traits>
#include <utility>

#include "../../include/diffrp_gb300.h"

namespace {

bool conv(PyObject* o, int& out) {
    const long v = PyLong_AsLong(o);
    if (v == -1 && PyErr_Occurred()) return false;
    if (v < INT32_MIN || v > INT32_MAX) {
        PyErr_SetString(PyExc_OverflowError, "int argument out of range");
        return false;
    }
    out = (int)v;
    return true;
}

bool conv(PyObject* o, unsigned& out) {
    const unsigned long v = PyLong_AsUnsignedLong(o);
    if (v == (unsigned long)-1 && PyErr_Occurred()) return false;
    if (v > 0xffffffffUL) {
        PyErr_SetString(PyExc_OverflowError, "unsigned argument out of range");
        return false;
    }
    out = (unsigned)v;
    return true;
}

bool conv(PyObject* o, long long& out) {
    out = PyLong_AsLongLong(o);
    return !(out == -1 && PyErr_Occurred());
}

bool conv(PyObject* o, unsigned long long& out) {
    out = PyLong_AsUnsignedLongLong(o);
    return !(out == (unsigned long long)-1 && PyErr_Occurred());
}

bool conv(PyObject* o, size_t& out) {
    out = PyLong_AsSize_t(o);
    return !(out == (size_t)-1 && PyErr_Occurred());
}

// Python float or int, or an object with a numeric .value (ctypes.c_float).
bool conv(PyObject* o, float& out) {
    if (PyFloat_Check(o) || PyLong_Check(o)) {
        const double d = PyFloat_AsDouble(o);
        if (d == -1.0 && PyErr_Occurred()) return false;
        out = (float)d;
        return true;
    }
    PyObject* v = PyObject_GetAttrString(o, "value");
    if (!v) return false;
    const double d = PyFloat_AsDouble(v);
    Py_DECREF(v);
    if (d == -1.0 && PyErr_Occurred()) return false;
    out = (float)d;
    return true;
}

// Pointers: None -> NULL, an int address, or (as ctypes accepts) an object
// whose _as_parameter_ or .value is one of those (c_void_p, stream wrappers).
template <typename T>
bool conv(PyObject* o, T*& out) {
    if (o == Py_None) {
        out = nullptr;
        return true;
    }
    if (!PyLong_Check(o)) {
        for (const char* attr : {"_as_parameter_", "value"}) {
            if (PyObject_HasAttrString(o, attr)) {
                PyObject* v = PyObject_GetAttrString(o, attr);
                if (!v) return false;
                const bool ok = v != o && conv(v, out);
                Py_DECREF(v);
                if (!ok && !PyErr_Occurred()) PyErr_SetString(PyExc_TypeError, "pointer argument expected");
                return ok;
            }
        }
        PyErr_SetString(PyExc_TypeError, "pointer argument expected (int, None or a ctypes pointer)");
        return false;
    }
    void* p = PyLong_AsVoidPtr(o);
    if (!p && PyErr_Occurred()) return false;
    out = reinterpret_cast<T*>(p);
    return true;
}

template <typename... Args, size_t... I>
PyObject* invoke_impl(int (*fn)(Args...), PyObject* const* argv, std::index_sequence<I...>) {
    std::tuple<std::remove_cv_t<Args>...> vals;
    const bool ok = (conv(argv[I], std::get<I>(vals)) && ...);
    if (!ok) return nullptr;
    int status;
    Py_BEGIN_ALLOW_THREADS
    status = fn(std::get<I>(vals)...);
    Py_END_ALLOW_THREADS
    return PyLong_FromLong(status);
}

template <typename... Args>
PyObject* invoke(int (*fn)(Args...), const char* name, PyObject* const* argv, Py_ssize_t nargs) {
    if (nargs != (Py_ssize_t)sizeof...(Args)) {
        PyErr_Format(PyExc_TypeError, "%s takes %d arguments (%zd given)", name, (int)sizeof...(Args), nargs);
        return nullptr;
    }
    return invoke_impl(fn, argv, std::index_sequence_for<Args...>{});
}

#define DRP_FAST(name)                                                              \
    PyObject* w_##name(PyObject*, PyObject* const* argv, Py_ssize_t nargs) {        \
        return invoke(&name, #name, argv, nargs);                                   \
    }
#define DRP_ENTRY(name) {#name, reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(w_##name)), \
                         METH_FASTCALL, nullptr}

// The per-call entry points of the drop-in ops, the loss and the batching
// form (workspace-size queries keep ctypes: they write through out-pointers
// and are cached by the caller).
DRP_FAST(drp_rasterize_fwd)
DRP_FAST(drp_rasterize_bwd)
DRP_FAST(drp_interpolate_fwd)
DRP_FAST(drp_interpolate_bwd)
DRP_FAST(drp_interpolate_sparse_fwd)
DRP_FAST(drp_interpolate_sparse_bwd)
DRP_FAST(drp_antialias_topology)
DRP_FAST(drp_antialias_fwd)
DRP_FAST(drp_antialias_bwd)
DRP_FAST(drp_edge_gradient_bwd)
DRP_FAST(drp_l1_loss_fwd)
DRP_FAST(drp_transform_points_fwd)
DRP_FAST(drp_transform_points_bwd)
DRP_FAST(drp_copy_async)
DRP_FAST(drp_batch_forward)
DRP_FAST(drp_batch_forward_l1)
DRP_FAST(drp_batch_forward_l1_grad)
DRP_FAST(drp_scale_floats)
DRP_FAST(drp_batch_backward)

PyMethodDef methods[] = {
    DRP_ENTRY(drp_rasterize_fwd),     DRP_ENTRY(drp_rasterize_bwd),       DRP_ENTRY(drp_interpolate_fwd),
    DRP_ENTRY(drp_interpolate_bwd),   DRP_ENTRY(drp_interpolate_sparse_fwd), DRP_ENTRY(drp_interpolate_sparse_bwd),
    DRP_ENTRY(drp_antialias_topology), DRP_ENTRY(drp_antialias_fwd),      DRP_ENTRY(drp_antialias_bwd),
    DRP_ENTRY(drp_edge_gradient_bwd), DRP_ENTRY(drp_l1_loss_fwd),         DRP_ENTRY(drp_batch_forward),
    DRP_ENTRY(drp_batch_forward_l1),  DRP_ENTRY(drp_batch_forward_l1_grad),  DRP_ENTRY(drp_scale_floats),  DRP_ENTRY(drp_batch_backward),      DRP_ENTRY(drp_transform_points_fwd),
    DRP_ENTRY(drp_transform_points_bwd), DRP_ENTRY(drp_copy_async), {nullptr, nullptr, 0, nullptr}};

PyModuleDef module = {PyModuleDef_HEAD_INIT, "_drp_fast", "CPython fast path onto libdiffrp_gb300", -1, methods,
                      nullptr, nullptr, nullptr, nullptr};

}  // namespace

PyMODINIT_FUNC PyInit__drp_fast(void) { return PyModule_Create(&module); }
