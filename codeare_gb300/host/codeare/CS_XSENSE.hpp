// CS_XSENSE.hpp -- compressed sensing over the GB300 NCSENSE operator with
// the interface of codeare's CS_XSENSE<T> (reference:
// src/matrix/ft/CS_XSENSE.hpp:47-431) for ft = 3 (NCSENSE) and ft = 2 (NFFT).
//
// Params keys as the reference constructor (CS_XSENSE.hpp:73-140) and its
// NLCG (src/optimisation/NLCG.hpp:33-40): tvw1, tv1, tvw2, tv2, xfmw, l1,
// pnorm, nlopt, ft, csiter, wl_family, wl_member, nliter, cgconv, lsiter,
// lsa, lsb, parallel_linesearch, verbose; the NCSENSE keys (sensitivities,
// nk, ftiter, fteps, cgiter, cgeps, lambda, alpha) or the NFFT keys (nk,
// imsz, m, alpha, maxit, epsilon) build the operator.
//
//   Trafo / operator*   E, the NCSENSE forward operator
//   Adjoint / ->*       the CS reconstruction: x0 = NCSENSE ->* data, TV
//                       weights scaled by max |x0|, csiter NLCG runs
//   obj, df             the objective and its gradient (CS_XSENSE.hpp:197-232)
// Every step runs on the GPU (libcgs.so cgs_cs_*).  Supported: ft = 3 and 2;
// nlopt 0 (NLCG) and 2 (Split Bregman, whose Minimise is empty in the
// reference); wl_family -1 (no wavelet).  Anything else throws, where the
// reference either throws as well or needs DFT / CSENSE / L-BFGS / DWT.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include <memory>

#include "NCSENSE.hpp"

template <class T> class CS_XSENSE : public FT<T> {
    typedef typename TypeTraits<T>::RT RT;

public:
    explicit CS_XSENSE(const Params &p) : FT<T>(p)
    {
        const int ft = try_to_fetch<int>(p, "ft", 4);
        if (ft == 3) m_ncs.reset(new NCSENSE<T>(p));
        else if (ft == 2) m_nft.reset(new NFFT<T>(p));
        else throw std::invalid_argument("CS_XSENSE: ft = 2 (NFFT) or 3 (NCSENSE) run on the GPU");
        cgs_cs_opts &o = m_o;
        o = cgs_cs_opts{};
        o.ft = ft;
        o.tvw[0] = try_to_fetch<float>(p, "tvw1", 0.f);
        o.tvw[1] = try_to_fetch<float>(p, "tvw2", 0.f);
        dims(p, "tv1", 0);
        dims(p, "tv2", 1);
        o.xfmw = try_to_fetch<float>(p, "xfmw", 0.f);
        o.l1 = try_to_fetch<float>(p, "l1", 0.f);
        o.pnorm = try_to_fetch<float>(p, "pnorm", 0.f);
        o.nlopt = try_to_fetch<int>(p, "nlopt", 0);
        o.csiter = try_to_fetch<int>(p, "csiter", 0);
        o.wl_family = try_to_fetch<int>(p, "wl_family", -1);
        if (o.wl_family < -1 || o.wl_family > 5) o.wl_family = -1;  // CS_XSENSE.hpp:131-132
        o.wl_member = try_to_fetch<int>(p, "wl_member", 0);
        o.nliter = try_to_fetch<int>(p, "nliter", 0);
        o.cgconv = try_to_fetch<float>(p, "cgconv", 0.f);
        o.lsiter = try_to_fetch<int>(p, "lsiter", 0);
        o.lsa = try_to_fetch<float>(p, "lsa", 0.f);
        o.lsb = try_to_fetch<float>(p, "lsb", 0.f);
        o.parallel_linesearch = try_to_fetch<bool>(p, "parallel_linesearch", false) ? 1 : 0;
        // the NCSENSE inverse: NCSENSE.hpp:69-184 defaults
        o.cgiter = (int)try_to_fetch<size_t>(p, "cgiter", 0);
        o.cgeps = try_to_fetch<double>(p, "cgeps", 1.0e-6);
        o.lambda = try_to_fetch<double>(p, "lambda", 1.0e-6);
        o.ftiter = (int)try_to_fetch<size_t>(p, "ftiter", 3);
        o.fteps = try_to_fetch<double>(p, "fteps", 1.0e-3);
        if (ft == 2) {  // NFFT::Adjoint's own settings (NFFT.hpp:114-115)
            o.ftiter = (int)try_to_fetch<size_t>(p, "maxit", 3);
            o.fteps = try_to_fetch<double>(p, "epsilon", 7.0e-4);
        }
    }

    CS_XSENSE(const CS_XSENSE &) = delete;
    CS_XSENSE &operator=(const CS_XSENSE &) = delete;
    virtual ~CS_XSENSE() { release(); }

    virtual void KSpace(const Matrix<RT> &k) { ft().KSpace(k); }
    virtual void Weights(const Matrix<RT> &w) { ft().Weights(w); }
    virtual void Sensitivities(const Matrix<T> &sm) { ft().Sensitivities(sm); }

    virtual Matrix<T> Trafo(const MatrixType<T> &m) const { return m_ncs ? m_ncs->Trafo(m) : m_nft->Trafo(m); }
    virtual Matrix<T> operator*(const MatrixType<T> &m) const { return Trafo(m); }

    virtual Matrix<T> Adjoint(const MatrixType<T> &m) const
    {
        Matrix<T> out(image_dims());
        m_rep = cgs_cs_report{};
        cgs_host::check(cgs_cs_adjoint(handle(), reinterpret_cast<const float *>(m.Ptr()),
                                       reinterpret_cast<float *>(out.Ptr()), &m_rep, nullptr),
                        "cgs_cs_adjoint");
        return out;
    }
    virtual Matrix<T> operator->*(const MatrixType<T> &m) const { return Adjoint(m); }

    // gradient of the objective at x for data y (CS_XSENSE::df with data = y)
    Matrix<T> df(const Matrix<T> &y, const Matrix<T> &x) const
    {
        Matrix<T> g(image_dims());
        cgs_host::check(cgs_cs_df(handle(), reinterpret_cast<const float *>(y.Ptr()),
                                  reinterpret_cast<const float *>(x.Ptr()), reinterpret_cast<float *>(g.Ptr()),
                                  nullptr),
                        "cgs_cs_df");
        return g;
    }

    // objective at x + t dx for data y; rmse = sqrt(data term / nnz(y))
    RT obj(const Matrix<T> &y, const Matrix<T> &x, const Matrix<T> &dx, const RT &t, RT &rmse) const
    {
        double o = 0.0, r = 0.0;
        cgs_host::check(cgs_cs_obj(handle(), reinterpret_cast<const float *>(y.Ptr()),
                                   reinterpret_cast<const float *>(x.Ptr()), reinterpret_cast<const float *>(dx.Ptr()),
                                   (float)t, &o, &r, nullptr),
                        "cgs_cs_obj");
        rmse = (RT)r;
        return (RT)o;
    }

    const cgs_cs_report &LastReport() const { return m_rep; }
    const FT<T> &getFT() const { return m_ncs ? (const FT<T> &)*m_ncs : (const FT<T> &)*m_nft; }

    virtual std::ostream &Print(std::ostream &os) const
    {
        Operator<T>::Print(os);
        os << "    Weights: TV(" << m_o.tvw[0] << ") TV(" << m_o.tvw[1] << ") XF(" << m_o.xfmw << ") L1(" << m_o.l1
           << ") Pnorm: " << m_o.pnorm << "\n";
        os << "    NLCG iterations: (" << m_o.nliter << ") LS(" << m_o.lsiter << ") conv(" << m_o.cgconv
           << ") lsa(" << m_o.lsa << ") lsb(" << m_o.lsb << ")\n";
        return getFT().Print(os);
    }

private:
    void dims(const Params &p, const char *key, int i)
    {
        m_o.ntvdims[i] = 0;
        if (!p.exists(key)) return;
        std::vector<size_t> v;
        try { v = p.Get<std::vector<size_t>>(key); } catch (const std::bad_any_cast &) { return; }
        for (size_t j = 0; j < v.size() && j < 3; ++j) m_o.tvdims[i][j] = (int)v[j];
        m_o.ntvdims[i] = (int)std::min<size_t>(v.size(), 3);
    }

    // created on first use: the plan needs k-space, weights and sensitivities
    cgs_cs *handle() const
    {
        if (!m_cs)
            cgs_host::check(cgs_cs_create(&m_cs, m_ncs ? m_ncs->Plan() : m_nft->Plan(), &m_o), "cgs_cs_create");
        return m_cs;
    }

    void release()
    {
        if (m_cs) cgs_cs_destroy(m_cs);
        m_cs = nullptr;
    }

    FT<T> &ft() { return m_ncs ? (FT<T> &)*m_ncs : (FT<T> &)*m_nft; }
    std::vector<size_t> image_dims() const { return m_ncs ? m_ncs->image_dims() : m_nft->image_dims(); }

    std::unique_ptr<NCSENSE<T>> m_ncs;
    std::unique_ptr<NFFT<T>> m_nft;
    cgs_cs_opts m_o{};
    mutable cgs_cs *m_cs = nullptr;
    mutable cgs_cs_report m_rep{};
};
