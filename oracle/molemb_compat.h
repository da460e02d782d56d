/*
 * Forced-include header for building the reference's own C_API/MolEmb.cpp,
 * unmodified and from its own source tree, against numpy 2 (oracle/_ref only).
 * numpy 2 dropped NPY_IN_ARRAY and its PyArray_DIM / PyArray_DATA accessors no
 * longer accept a PyObject*; these wrappers restore both so the untouched
 * source compiles. This is test infrastructure: nothing in the product uses it.
 */
#include <Python.h>
#include <numpy/arrayobject.h>
#define NPY_IN_ARRAY NPY_ARRAY_IN_ARRAY
#undef PyArray_DIM
#define PyArray_DIM(obj, n) (PyArray_DIMS((PyArrayObject *)(obj))[n])
static inline void *tm_compat_array_data(void *obj) {
  return PyArray_DATA((PyArrayObject *)obj);
}
#define PyArray_DATA(obj) tm_compat_array_data((void *)(obj))
