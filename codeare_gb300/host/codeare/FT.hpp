// FT.hpp -- operator bases (reference: src/matrix/Operator.hpp:14-32 and
// src/matrix/ft/FT.hpp:31-138).  Operator<T>: operator*, operator->*,
// operator/; FT<T> adds Trafo / Adjoint and the trajectory setters.
#pragma once

#include <ostream>
#include <typeinfo>

#include "Matrix.hpp"
#include "Params.hpp"

template <class T> class Operator {
public:
    typedef typename TypeTraits<T>::RT RT;
    Operator() {}
    virtual ~Operator() {}
    virtual Matrix<T> operator*(const MatrixType<T> &) const { return Matrix<T>(); }
    virtual Matrix<T> operator->*(const MatrixType<T> &) const { return Matrix<T>(); }
    virtual Matrix<T> operator/(const MatrixType<T> &) const { return Matrix<T>(); }
    virtual std::ostream &Print(std::ostream &os) const { return os << "  " << typeid(*this).name() << std::endl; }
    friend std::ostream &operator<<(std::ostream &os, const Operator<T> &o) { return o.Print(os); }
};

template <class T> class FT : public Operator<T> {
public:
    typedef typename TypeTraits<T>::RT RT;
    FT() {}
    explicit FT(const Params &p) : m_params(p) {}
    virtual ~FT() {}
    virtual Matrix<T> Trafo(const MatrixType<T> &) const { return Matrix<T>(); }
    virtual Matrix<T> Adjoint(const MatrixType<T> &) const { return Matrix<T>(); }
    virtual Matrix<T> operator*(const MatrixType<T> &m) const { return Trafo(m); }
    virtual Matrix<T> operator->*(const MatrixType<T> &m) const { return Adjoint(m); }
    virtual void KSpace(const Matrix<RT> &) {}
    virtual void Weights(const Matrix<RT> &) {}
    virtual void Sensitivities(const Matrix<T> &) {}
    virtual void Mask(const Matrix<RT> &) {}

protected:
    Params m_params;
};
