// Matrix.hpp -- the subset of codeare's column-major N-d Matrix<T> that the
// CG-SENSE path and its plugin use (reference: src/matrix/Matrix.hpp:165-200,
// size/numel/ndims helpers, squeeze at src/matrix/Algos.hpp:933).  First index
// fastest; storage contiguous.  Element-wise arithmetic is limited to what the
// host CG loop (CGLS.hpp) needs.
#pragma once

#include <algorithm>
#include <cassert>
#include <complex>
#include <cstddef>
#include <numeric>
#include <stdexcept>
#include <vector>

typedef std::complex<float> cxfl;
typedef std::complex<double> cxdb;

template <class T> struct TypeTraits { typedef T RT; };
template <class T> struct TypeTraits<std::complex<T>> { typedef T RT; };

template <class T> class Matrix {
public:
    typedef T value_type;

    Matrix() : _dim(2, 1), _data(1, T(0)) {}
    // Matrix(n) is an n x n matrix, as in codeare
    explicit Matrix(size_t n) : _dim{n, n}, _data(n * n, T(0)) {}
    Matrix(size_t m, size_t n) : _dim{m, n}, _data(m * n, T(0)) {}
    Matrix(size_t m, size_t n, size_t k) : _dim{m, n, k}, _data(m * n * k, T(0)) {}
    Matrix(size_t m, size_t n, size_t k, size_t l) : _dim{m, n, k, l}, _data(m * n * k * l, T(0)) {}
    explicit Matrix(const std::vector<size_t> &dims) : _dim(dims)
    {
        if (_dim.empty()) _dim = {1, 1};
        if (_dim.size() == 1) _dim.push_back(1);
        _data.assign(prod(), T(0));
    }

    size_t Size() const { return _data.size(); }
    size_t NDim() const { return _dim.size(); }
    size_t Dim(size_t i) const { return i < _dim.size() ? _dim[i] : 1; }
    const std::vector<size_t> &Dim() const { return _dim; }

    T &operator[](size_t i) { return _data[i]; }
    const T &operator[](size_t i) const { return _data[i]; }
    T &operator()(size_t i) { return _data[i]; }
    const T &operator()(size_t i) const { return _data[i]; }
    T &operator()(size_t i, size_t j) { return _data[i + _dim[0] * j]; }
    const T &operator()(size_t i, size_t j) const { return _data[i + _dim[0] * j]; }
    T &operator()(size_t i, size_t j, size_t k) { return _data[i + _dim[0] * (j + _dim[1] * k)]; }
    const T &operator()(size_t i, size_t j, size_t k) const { return _data[i + _dim[0] * (j + _dim[1] * k)]; }

    T *Ptr() { return _data.data(); }
    const T *Ptr() const { return _data.data(); }
    typename std::vector<T>::iterator Begin() { return _data.begin(); }
    typename std::vector<T>::iterator End() { return _data.end(); }
    typename std::vector<T>::const_iterator Begin() const { return _data.begin(); }
    typename std::vector<T>::const_iterator End() const { return _data.end(); }
    std::vector<T> &Container() { return _data; }
    const std::vector<T> &Container() const { return _data; }

    // element-wise arithmetic used by the host CG loop
    Matrix &operator+=(const Matrix &o) { check(o); for (size_t i = 0; i < Size(); ++i) _data[i] += o._data[i]; return *this; }
    Matrix &operator-=(const Matrix &o) { check(o); for (size_t i = 0; i < Size(); ++i) _data[i] -= o._data[i]; return *this; }
    template <class S> Matrix &operator*=(const S &s) { for (auto &v : _data) v *= s; return *this; }
    Matrix operator+(const Matrix &o) const { Matrix r(*this); r += o; return r; }
    Matrix operator-(const Matrix &o) const { Matrix r(*this); r -= o; return r; }
    template <class S> Matrix operator*(const S &s) const { Matrix r(*this); r *= s; return r; }
    friend Matrix operator*(const typename TypeTraits<T>::RT &s, const Matrix &m) { return m * s; }

    void Reshape(const std::vector<size_t> &dims)
    {
        size_t p = 1;
        for (size_t d : dims) p *= d;
        if (p != Size()) throw std::invalid_argument("Reshape: element count differs");
        _dim = dims;
    }

private:
    size_t prod() const { size_t p = 1; for (size_t d : _dim) p *= d; return p; }
    void check(const Matrix &o) const { if (o.Size() != Size()) throw std::invalid_argument("size mismatch"); }
    std::vector<size_t> _dim;
    std::vector<T> _data;
};

template <class T> using MatrixType = Matrix<T>;

template <class T> inline size_t numel(const Matrix<T> &m) { return m.Size(); }
template <class T> inline size_t size(const Matrix<T> &m, size_t d) { return m.Dim(d); }
template <class T> inline std::vector<size_t> size(const Matrix<T> &m) { return m.Dim(); }

// number of dimensions without trailing singletons (codeare's ndims)
template <class T> inline size_t ndims(const Matrix<T> &m)
{
    size_t n = m.NDim();
    while (n > 2 && m.Dim(n - 1) == 1) --n;
    return n;
}

// drop singleton dimensions (codeare's squeeze keeps at least 2)
template <class T> inline Matrix<T> squeeze(const Matrix<T> &m)
{
    std::vector<size_t> d;
    for (size_t v : m.Dim())
        if (v != 1) d.push_back(v);
    while (d.size() < 2) d.push_back(1);
    Matrix<T> r(m);
    r.Reshape(d);
    return r;
}

template <class T> inline Matrix<T> zeros(const std::vector<size_t> &dims) { return Matrix<T>(dims); }

// Re <a, b> with FP64 accumulation (the reference accumulates in complex<float>,
// src/matrix/linalg/Lapack.hpp:619-624)
template <class T> inline T dotc(const Matrix<T> &a, const Matrix<T> &b)
{
    std::complex<double> s = 0;
    for (size_t i = 0; i < a.Size(); ++i) s += std::conj(std::complex<double>(a[i])) * std::complex<double>(b[i]);
    return T((typename TypeTraits<T>::RT)s.real(), (typename TypeTraits<T>::RT)s.imag());
}
