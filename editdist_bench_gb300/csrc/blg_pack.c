/*
 * _blgpack: native packing of Python str/bytes sequences into bitlev's
 * packed layout (one byte buffer + int64 offsets off[0..n], string i =
 * buf[off[i] .. off[i+1])), the input format of the C-ABI.
 *
 * Rules of the reference's packer (csrc/edpy.c:14-35, 200-224): a str must be
 * of the 1-byte kind (code points <= U+00FF; 1 character = 1 byte), else
 * ValueError; bytes are taken as they are; any other item is a TypeError.
 * The buffer is never empty (one zero byte for an all-empty set).
 *
 *   size(seq)                  -> (n, total_bytes)   validation pass
 *   pack_into(seq, buf_addr, buf_cap, off_addr)      one memcpy per string into
 *                                 caller memory (e.g. page-locked staging);
 *                                 off_addr receives n+1 int64 offsets
 *
 * The Python layer (editdist_bench_gb300/_common.py) allocates the arrays;
 * this module only reads the items and copies their bytes, with the GIL held
 * (the items are Python objects).
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdint.h>
#include <string.h>

/* the messages of the Python layer (editdist_bench_gb300/_common.py) */
static const char *WIDE_MSG = "string has characters above U+00FF; pass bytes (e.g. UTF-8 encoded) instead";
static const char *TYPE_MSG = "expected str or bytes";

/* Pointer and length of one item, or -1 with an exception set. */
static int item_bytes(PyObject *o, const char **p, Py_ssize_t *len) {
    if (PyUnicode_Check(o)) {
        if (PyUnicode_KIND(o) != PyUnicode_1BYTE_KIND) {
            PyErr_SetString(PyExc_ValueError, WIDE_MSG);
            return -1;
        }
        *p = (const char *)PyUnicode_1BYTE_DATA(o);
        *len = PyUnicode_GET_LENGTH(o);
        return 0;
    }
    if (PyBytes_Check(o)) {
        *p = PyBytes_AS_STRING(o);
        *len = PyBytes_GET_SIZE(o);
        return 0;
    }
    PyErr_SetString(PyExc_TypeError, TYPE_MSG);
    return -1;
}

static PyObject *py_size(PyObject *self, PyObject *arg) {
    (void)self;
    PyObject *seq = PySequence_Fast(arg, "expected a sequence");
    if (!seq) return NULL;
    const Py_ssize_t n = PySequence_Fast_GET_SIZE(seq);
    PyObject **items = PySequence_Fast_ITEMS(seq);
    long long total = 0;
    for (Py_ssize_t i = 0; i < n; i++) {
        const char *p;
        Py_ssize_t len;
        if (item_bytes(items[i], &p, &len)) {
            Py_DECREF(seq);
            return NULL;
        }
        total += len;
    }
    Py_DECREF(seq);
    return Py_BuildValue("(nL)", n, total);
}

static PyObject *py_pack_into(PyObject *self, PyObject *args) {
    (void)self;
    PyObject *arg;
    unsigned long long buf_addr, off_addr;
    long long cap;
    if (!PyArg_ParseTuple(args, "OKLK", &arg, &buf_addr, &cap, &off_addr)) return NULL;
    PyObject *seq = PySequence_Fast(arg, "expected a sequence");
    if (!seq) return NULL;
    const Py_ssize_t n = PySequence_Fast_GET_SIZE(seq);
    PyObject **items = PySequence_Fast_ITEMS(seq);
    uint8_t *buf = (uint8_t *)(uintptr_t)buf_addr;
    int64_t *off = (int64_t *)(uintptr_t)off_addr;
    long long at = 0;
    off[0] = 0;
    for (Py_ssize_t i = 0; i < n; i++) {
        const char *p;
        Py_ssize_t len;
        if (item_bytes(items[i], &p, &len)) {
            Py_DECREF(seq);
            return NULL;
        }
        if (at + len > cap) {
            Py_DECREF(seq);
            PyErr_SetString(PyExc_ValueError, "packed buffer too small");
            return NULL;
        }
        memcpy(buf + at, p, (size_t)len);
        at += len;
        off[i + 1] = at;
    }
    Py_DECREF(seq);
    if (at == 0 && cap > 0) buf[0] = 0;       /* never empty */
    return PyLong_FromLongLong(at);
}

static PyMethodDef methods[] = {
    {"size", py_size, METH_O, "(n, total bytes) of a str/bytes sequence, validating every item"},
    {"pack_into", py_pack_into, METH_VARARGS, "pack_into(seq, buf_addr, buf_cap, off_addr) -> bytes written"},
    {NULL, NULL, 0, NULL},
};

static struct PyModuleDef module = {PyModuleDef_HEAD_INIT, "_blgpack", "native packing of str/bytes sequences",
                                    -1, methods, NULL, NULL, NULL, NULL};

PyMODINIT_FUNC PyInit__blgpack(void) { return PyModule_Create(&module); }
