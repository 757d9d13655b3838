// CGLS.hpp -- host CG over any Operator<T> (reference:
// src/optimisation/CGLS.hpp:30-59): p = A/b; r = p; rn = xn = Re<r,p>; per
// iteration res = rn/xn, stop on NaN or res <= eps; q = A/(A*p) + lambda p;
// ts = rn/Re<p,q>; x += ts p; r -= ts q; p = r + (rn_new/rn) p.  The scalars
// accumulate in FP64 (the reference uses complex<float>).  NCSENSE::Adjoint
// does not come here: it runs the same loop fused on the GPU (cgs_solve).
#pragma once

#include <cmath>
#include <cstdio>
#include <vector>

#include "FT.hpp"

namespace codeare {
namespace optimisation {

template <class T> class CGLS {
    typedef typename TypeTraits<T>::RT RT;

public:
    CGLS(const size_t &maxit = 10, const RT &epsilon = 1.0e-6, const RT &lambda = 1.0e-6, const int &verbosity = 0)
        : _maxit(maxit), _epsilon(epsilon), _lambda(lambda), _verbosity(verbosity) {}

    Matrix<T> Solve(const Operator<T> &A, const MatrixType<T> &b)
    {
        _res.clear();
        Matrix<T> p = A / b;
        if (_maxit == 0) return p;
        Matrix<T> r = p;
        double rn = std::real(std::complex<double>(dotc(r, p))), xn = rn;
        Matrix<T> x(p.Dim());
        for (size_t i = 0; i < _maxit; ++i) {
            _res.push_back(rn / xn);
            if (std::isnan(_res[i]) || _res[i] <= _epsilon) {
                std::printf("    %03zu %.7f\n", i, _res[i]);
                break;
            }
            if (_verbosity) std::printf("    %03zu %.7f\n", i, _res[i]);
            Matrix<T> q = A / (A * p);
            if (_lambda != RT(0)) q += p * _lambda;
            const RT ts = (RT)(rn / std::real(std::complex<double>(dotc(p, q))));
            x += p * ts;
            r -= q * ts;
            const double rno = rn;
            rn = std::real(std::complex<double>(dotc(r, r)));
            p *= (RT)(rn / rno);
            p += r;
        }
        return x;
    }

    const std::vector<double> &Residuals() const { return _res; }

private:
    size_t _maxit;
    RT _epsilon, _lambda;
    int _verbosity;
    std::vector<double> _res;
};

}  // namespace optimisation
}  // namespace codeare
