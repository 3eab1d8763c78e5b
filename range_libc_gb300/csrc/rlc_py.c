/* _rlcfast -- CPython entry points for the per-call host-buffer methods of
 * range_libc_gb300.range_libc (the role the reference's Cython module plays).
 *
 * Each function takes a method handle (as an integer) and numpy arrays,
 * checks them through the buffer protocol and calls the C ABI directly.  It
 * returns the C ABI status, or -1 when an argument is not a C-contiguous
 * buffer of the expected item type, rank and length, in which case the
 * Python layer repeats the call through its own argument checks (which raise
 * the reference's errors).  Nothing here computes a range.
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>

#include "rangelibc.h"

#include <string.h>

/* a C-contiguous buffer of `fmt` items ("f" float32, "d" float64) of rank `ndim` */
static int get_buf(PyObject* o, Py_buffer* v, const char* fmt, int ndim, int writable) {
    int flags = PyBUF_C_CONTIGUOUS | PyBUF_FORMAT | (writable ? PyBUF_WRITABLE : 0);
    if (PyObject_GetBuffer(o, v, flags) != 0) {
        PyErr_Clear();
        return -1;
    }
    const char* f = v->format ? v->format : "B";
    if (f[0] == '=' || f[0] == '<' || f[0] == '@') ++f;   /* native little-endian */
    if (strcmp(f, fmt) != 0 || v->ndim != ndim) {
        PyBuffer_Release(v);
        return -1;
    }
    return 0;
}

static PyObject* fused(PyObject* self, PyObject* args) {
    (void)self;
    unsigned long long h;
    PyObject *oi, *oa, *oo, *ow;
    if (!PyArg_ParseTuple(args, "KOOOO", &h, &oi, &oa, &oo, &ow)) return NULL;
    Py_buffer bi, ba, bo, bw;
    if (get_buf(oi, &bi, "f", 2, 0)) return PyLong_FromLong(-1);
    if (get_buf(oa, &ba, "f", 1, 0)) { PyBuffer_Release(&bi); return PyLong_FromLong(-1); }
    if (get_buf(oo, &bo, "f", 1, 0)) { PyBuffer_Release(&bi); PyBuffer_Release(&ba); return PyLong_FromLong(-1); }
    if (get_buf(ow, &bw, "d", 1, 1)) {
        PyBuffer_Release(&bi); PyBuffer_Release(&ba); PyBuffer_Release(&bo);
        return PyLong_FromLong(-1);
    }
    int rc = -1;
    const Py_ssize_t n = bi.shape[0], na = ba.shape[0];
    if (bi.shape[1] == 3 && bo.shape[0] >= na && bw.shape[0] >= n && n <= 0x7fffffff && na <= 0x7fffffff) {
        Py_BEGIN_ALLOW_THREADS
        rc = rlc_calc_range_repeat_angles_eval_sensor_model((rlc_method*)(uintptr_t)h, (const float*)bi.buf,
                                                             (const float*)ba.buf, (const float*)bo.buf,
                                                             (double*)bw.buf, (int)n, (int)na, 0, NULL);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&bi); PyBuffer_Release(&ba); PyBuffer_Release(&bo); PyBuffer_Release(&bw);
    return PyLong_FromLong(rc);
}

static PyObject* repeat_angles(PyObject* self, PyObject* args) {
    (void)self;
    unsigned long long h;
    PyObject *oi, *oa, *oo;
    if (!PyArg_ParseTuple(args, "KOOO", &h, &oi, &oa, &oo)) return NULL;
    Py_buffer bi, ba, bo;
    if (get_buf(oi, &bi, "f", 2, 0)) return PyLong_FromLong(-1);
    if (get_buf(oa, &ba, "f", 1, 0)) { PyBuffer_Release(&bi); return PyLong_FromLong(-1); }
    if (get_buf(oo, &bo, "f", 1, 1)) { PyBuffer_Release(&bi); PyBuffer_Release(&ba); return PyLong_FromLong(-1); }
    int rc = -1;
    const Py_ssize_t n = bi.shape[0], na = ba.shape[0];
    if (bi.shape[1] == 3 && bo.shape[0] >= n * na && n <= 0x7fffffff && na <= 0x7fffffff) {
        Py_BEGIN_ALLOW_THREADS
        rc = rlc_calc_range_repeat_angles((rlc_method*)(uintptr_t)h, (const float*)bi.buf, (const float*)ba.buf,
                                          (float*)bo.buf, (int)n, (int)na, 0, NULL);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&bi); PyBuffer_Release(&ba); PyBuffer_Release(&bo);
    return PyLong_FromLong(rc);
}

static PyObject* calc_range_many(PyObject* self, PyObject* args) {
    (void)self;
    unsigned long long h;
    PyObject *oi, *oo;
    if (!PyArg_ParseTuple(args, "KOO", &h, &oi, &oo)) return NULL;
    Py_buffer bi, bo;
    if (get_buf(oi, &bi, "f", 2, 0)) return PyLong_FromLong(-1);
    if (get_buf(oo, &bo, "f", 1, 1)) { PyBuffer_Release(&bi); return PyLong_FromLong(-1); }
    int rc = -1;
    const Py_ssize_t n = bo.shape[0];   /* the reference takes the count from outs */
    if (bi.shape[1] == 3 && bi.shape[0] >= n && n <= 0x7fffffff) {
        Py_BEGIN_ALLOW_THREADS
        rc = rlc_calc_range_many((rlc_method*)(uintptr_t)h, (const float*)bi.buf, (float*)bo.buf, (int)n, 0, NULL);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&bi); PyBuffer_Release(&bo);
    return PyLong_FromLong(rc);
}

static PyObject* eval_sensor_model(PyObject* self, PyObject* args) {
    (void)self;
    unsigned long long h;
    PyObject *oo, *orr, *ow;
    int nr, np_;
    if (!PyArg_ParseTuple(args, "KOOOii", &h, &oo, &orr, &ow, &nr, &np_)) return NULL;
    Py_buffer bo, br, bw;
    if (get_buf(oo, &bo, "f", 1, 0)) return PyLong_FromLong(-1);
    if (get_buf(orr, &br, "f", 1, 0)) { PyBuffer_Release(&bo); return PyLong_FromLong(-1); }
    if (get_buf(ow, &bw, "d", 1, 1)) { PyBuffer_Release(&bo); PyBuffer_Release(&br); return PyLong_FromLong(-1); }
    int rc = -1;
    if (nr >= 0 && np_ >= 0 && bo.shape[0] >= nr && br.shape[0] >= (Py_ssize_t)nr * np_ && bw.shape[0] >= np_) {
        Py_BEGIN_ALLOW_THREADS
        rc = rlc_eval_sensor_model((rlc_method*)(uintptr_t)h, (const float*)bo.buf, (const float*)br.buf,
                                   (double*)bw.buf, nr, np_, 0, NULL);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&bo); PyBuffer_Release(&br); PyBuffer_Release(&bw);
    return PyLong_FromLong(rc);
}

static PyMethodDef kMethods[] = {
    {"fused", fused, METH_VARARGS, "calc_range_repeat_angles_eval_sensor_model on host buffers"},
    {"repeat_angles", repeat_angles, METH_VARARGS, "calc_range_repeat_angles on host buffers"},
    {"calc_range_many", calc_range_many, METH_VARARGS, "calc_range_many on host buffers"},
    {"eval_sensor_model", eval_sensor_model, METH_VARARGS, "eval_sensor_model on host buffers"},
    {NULL, NULL, 0, NULL},
};

static struct PyModuleDef kModule = {PyModuleDef_HEAD_INIT, "_rlcfast", NULL, -1, kMethods, NULL, NULL, NULL, NULL};

PyMODINIT_FUNC PyInit__rlcfast(void) { return PyModule_Create(&kModule); }
