// Stand-in for the header of the adpy runtime (an empty git submodule in the reference,
// adFVM/cpp/include/mesh.hpp:4 includes it). It provides just what the reference's mesh
// builder sources (adFVM/cpp/cmesh.cpp, adFVM/cpp/mesh.cpp) use, so that those files compile
// UNMODIFIED into a Python extension that serves as the geometry oracle:
//   * arrType<T, shape1, shape2>: row-major array with (i), (i,j), (i,j,k) element access,
//     a (n, zero) constructor and move semantics,
//   * getArray / putArray between arrType and numpy arrays,
//   * the Python-2 C-API names used by the sources, mapped to their Python-3 equivalents,
//   * GET_MODULE / VALUE token-pasting helpers for the module init function.
// Written from the usage in those two files; no adpy code is reproduced. Test
// infrastructure only.
#ifndef INTERFACE_HPP
#define INTERFACE_HPP

#define PY_SSIZE_T_CLEAN
#include <Python.h>
#define PY_ARRAY_UNIQUE_SYMBOL afvm_refshim_ARRAY_API
#define NPY_NO_DEPRECATED_API NPY_1_7_API_VERSION
#include <numpy/arrayobject.h>

#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <map>
#include <string>
#include <utility>
#include <vector>

using namespace std;

#ifdef CPU_FLOAT32
typedef float scalar;
#define NPY_SCALAR NPY_FLOAT32
#else
typedef double scalar;
#define NPY_SCALAR NPY_FLOAT64
#endif
typedef int32_t integer;

#define PY3
#define PyInt_AsLong PyLong_AsLong
#define PyInt_Check PyLong_Check
#define PyString_Check PyUnicode_Check
#define PyString_AsString PyUnicode_AsUTF8
#define AFVM_SHIM_CAT(a, b) a##b
#define GET_MODULE(a, b) AFVM_SHIM_CAT(a, b)
#define AFVM_SHIM_STR(x) #x
#define VALUE(x) AFVM_SHIM_STR(x)

template <typename dtype, integer shape1 = 1, integer shape2 = 1>
class arrType {
  public:
    dtype* data;
    integer shape;
    bool ownData;

    arrType() : data(nullptr), shape(0), ownData(false) {}
    explicit arrType(integer n, bool zero = false) : shape(n), ownData(true) {
        data = new dtype[(size_t)n * shape1 * shape2];
        if (zero) memset(data, 0, sizeof(dtype) * (size_t)n * shape1 * shape2);
    }
    arrType(const arrType&) = delete;
    arrType& operator=(const arrType&) = delete;
    arrType(arrType&& o) noexcept : data(o.data), shape(o.shape), ownData(o.ownData) {
        o.data = nullptr; o.ownData = false; o.shape = 0;
    }
    arrType& operator=(arrType&& o) noexcept {
        if (this != &o) {
            release();
            data = o.data; shape = o.shape; ownData = o.ownData;
            o.data = nullptr; o.ownData = false; o.shape = 0;
        }
        return *this;
    }
    ~arrType() { release(); }
    void release() {
        if (ownData && data) delete[] data;
        data = nullptr; ownData = false;
    }
    dtype& operator()(integer i) { return data[(size_t)i * shape1 * shape2]; }
    dtype& operator()(integer i, integer j) { return data[(size_t)i * shape1 * shape2 + (size_t)j * shape2]; }
    dtype& operator()(integer i, integer j, integer k) {
        return data[(size_t)i * shape1 * shape2 + (size_t)j * shape2 + k];
    }
};

template <typename dtype, integer shape1 = 1, integer shape2 = 1>
class extArrType : public arrType<dtype, shape1, shape2> {};

typedef arrType<scalar> vec;
typedef arrType<scalar, 3> mat;
typedef arrType<integer> ivec;
typedef extArrType<scalar> ext_vec;

template <typename dtype> inline int npy_type_of();
template <> inline int npy_type_of<double>() { return NPY_FLOAT64; }
template <> inline int npy_type_of<float>() { return NPY_FLOAT32; }
template <> inline int npy_type_of<integer>() { return NPY_INT32; }

// borrow the numpy buffer (the Python object keeps it alive)
template <typename dtype, integer shape1, integer shape2>
void getArray(PyArrayObject* array, arrType<dtype, shape1, shape2>& tmp) {
    assert(array != NULL);
    assert(PyArray_IS_C_CONTIGUOUS(array));
    assert(PyArray_ITEMSIZE(array) == sizeof(dtype));
    tmp.release();
    tmp.data = (dtype*)PyArray_DATA(array);
    tmp.shape = (integer)PyArray_DIM(array, 0);
    tmp.ownData = false;
}

// copy into a new numpy array of shape (n[, shape1[, shape2]])
template <typename dtype, integer shape1, integer shape2>
PyObject* putArray(arrType<dtype, shape1, shape2>& tmp) {
    npy_intp dims[3] = {tmp.shape, shape1, shape2};
    int nd = 1;
    if (shape2 > 1) nd = 3;
    else if (shape1 > 1) nd = 2;
    PyObject* arr = PyArray_SimpleNew(nd, dims, npy_type_of<dtype>());
    memcpy(PyArray_DATA((PyArrayObject*)arr), tmp.data, sizeof(dtype) * (size_t)tmp.shape * shape1 * shape2);
    return arr;
}

#endif
