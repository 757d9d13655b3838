// NFFT.hpp -- GB300 NFFT operator with the interface of codeare's NFFT<T>
// (reference: src/matrix/ft/NFFT.hpp:36-511).  Construction from Params with
// the same keys and defaults (nk, imsz, m = 1, alpha = 1, epsilon = 7e-4,
// maxit = 3; NFFT.hpp:66-191), KSpace / Weights setters (:258-296), Trafo =
// forward NFFT (:305-361) and Adjoint = the CGNR inverse NFFT (:370-436).
// All arithmetic runs in libcgs.so on the GPU through the C ABI.  Not
// supported (the constructor throws): b0 / timing (the
// off-resonance plan) and pc.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "FT.hpp"
#include "../../../include/cgs.h"

namespace cgs_host {
inline void check(cgs_status s, const char *what)
{
    if (s != CGS_OK) throw std::runtime_error(std::string(what) + ": " + cgs_last_error());
}
}  // namespace cgs_host

template <class T> class NFFT : public FT<T> {
    typedef typename TypeTraits<T>::RT RT;
    static_assert(sizeof(T) == 8, "NFFT<T> is instantiated for complex<float>");

public:
    NFFT() {}

    explicit NFFT(const Params &p) : FT<T>(p)
    {
        if (!p.exists("nk")) throw std::invalid_argument("NFFT: number of k-space samples (nk) needs to be specified");
        m_M = unsigned_cast(p["nk"]);
        if (!p.exists("imsz")) throw std::invalid_argument("NFFT: image dimensions (imsz) need to be specified");
        m_N = p.Get<std::vector<size_t>>("imsz");
        // Cartesian third dimension (NFFT.hpp:85, 100-103): the last image
        // dimension is a stack of m_ncart slices, each a 2-D NFFT with the shared
        // trajectory (the reference leaves the FFT along the stack commented
        // out, :312-332, :412-432); here the slices are the plan's coils
        if (try_to_fetch<bool>(p, "3rd_dim_cart", false)) {
            if (m_N.size() != 3) throw std::invalid_argument("NFFT: 3rd_dim_cart needs a 3-D image size");
            m_ncart = m_N.back();
            m_N.pop_back();
        }
        // off-resonance data only takes effect when its size matches the image
        // (NFFT.hpp:113-140 of the reference warns and ignores it otherwise)
        size_t nimg = 1;
        for (size_t v : m_N) nimg *= v;
        if (p.exists("b0")) {
            bool fits = false;
            try { fits = p.Get<Matrix<RT>>("b0").Size() == nimg; } catch (...) {}
            if (fits) throw std::invalid_argument("NFFT: off-resonance correction (b0) is not supported");
            std::printf("  WARNING - NFFT: b0 field does not fit to image space. Defaulting to flat b0 = 0\n");
        }
        if (p.exists("pc")) throw std::invalid_argument("NFFT: phase correction (pc) is not supported");
        m_m = try_to_fetch<size_t>(p, "m", 1);
        m_alpha = try_to_fetch<float>(p, "alpha", 1.0f);
        m_epsilon = try_to_fetch<float>(p, "epsilon", 7.0e-4f);
        m_maxit = try_to_fetch<size_t>(p, "maxit", 3);
        plan();
    }

    NFFT(const NFFT &o) : FT<T>(o) { *this = o; }

    NFFT &operator=(const NFFT &o)
    {
        if (this == &o) return *this;
        release();
        this->m_params = o.m_params;
        m_N = o.m_N; m_M = o.m_M; m_m = o.m_m; m_alpha = o.m_alpha; m_epsilon = o.m_epsilon;
        m_maxit = o.m_maxit; m_k = o.m_k; m_w = o.m_w; m_ncart = o.m_ncart;
        m_have_k = o.m_have_k; m_have_w = o.m_have_w;
        if (!m_N.empty()) {
            plan();
            if (m_have_k) KSpace(m_k);
            if (m_have_w) Weights(m_w);
        }
        return *this;
    }

    NFFT(NFFT &&o) noexcept : FT<T>(o) { steal(o); }
    NFFT &operator=(NFFT &&o) noexcept
    {
        if (this != &o) { release(); this->m_params = o.m_params; steal(o); }
        return *this;
    }

    virtual ~NFFT() { release(); }

    virtual void KSpace(const Matrix<RT> &k)
    {
        // a per-slice trajectory (rank x nk x slices) only sets a flag in the
        // reference and never reaches the plan (NFFT.hpp:269-270): not accepted
        if (k.Size() != m_M * m_N.size())
            throw std::invalid_argument("NFFT: k-space must hold rank x nk values");
        m_k = k;
        cgs_host::check(cgs_set_kspace(m_plan, k.Ptr()), "cgs_set_kspace");
        m_have_k = true;
        if (m_have_w) cgs_host::check(cgs_set_weights(m_plan, m_w.Ptr()), "cgs_set_weights");
    }

    virtual void Weights(const Matrix<RT> &w)
    {
        if (w.Size() != m_M) throw std::invalid_argument("NFFT: weights must hold nk values");
        m_w = w;
        m_have_w = true;
        if (m_have_k) cgs_host::check(cgs_set_weights(m_plan, w.Ptr()), "cgs_set_weights");
    }

    virtual Matrix<T> Trafo(const MatrixType<T> &m) const
    {
        need_k();
        if (m.Size() != image_numel() * m_ncart) throw std::invalid_argument("NFFT::Trafo: image size mismatch");
        Matrix<T> out(m_M, m_ncart);
        cgs_host::check(cgs_nfft_trafo(m_plan, reinterpret_cast<const float *>(m.Ptr()),
                                       reinterpret_cast<float *>(out.Ptr()), nullptr), "cgs_nfft_trafo");
        return squeeze(out);
    }

    // iterative inverse NFFT (CGNR, maxit steps, epsilon threshold) as the reference's Adjoint
    virtual Matrix<T> Adjoint(const MatrixType<T> &m) const
    {
        need_k();
        if (m.Size() != m_M * m_ncart) throw std::invalid_argument("NFFT::Adjoint: sample count mismatch");
        if (!m_have_w) {
            // the reference's solver reads uninitialised weights here; use unit weights
            Matrix<RT> ones(m_M, 1);
            for (auto &v : ones.Container()) v = 1.f;
            const_cast<NFFT *>(this)->Weights(ones);
        }
        Matrix<T> out(out_dims());
        cgs_host::check(cgs_nfft_itrafo(m_plan, reinterpret_cast<const float *>(m.Ptr()),
                                        reinterpret_cast<float *>(out.Ptr()), (int)m_maxit, (double)m_epsilon,
                                        nullptr), "cgs_nfft_itrafo");
        return out;
    }

    // the true adjoint A^H (no iteration); no reference counterpart as a method
    Matrix<T> AdjointTrue(const MatrixType<T> &m) const
    {
        need_k();
        Matrix<T> out(out_dims());
        cgs_host::check(cgs_nfft_adjoint(m_plan, reinterpret_cast<const float *>(m.Ptr()),
                                         reinterpret_cast<float *>(out.Ptr()), nullptr), "cgs_nfft_adjoint");
        return out;
    }

    size_t Rank() const { return m_N.size(); }
    size_t ImageSize() const { return m_N.empty() ? 0 : m_N[0]; }
    const std::vector<size_t> &image_dims() const { return m_N; }
    cgs_plan *Plan() const { return m_plan; }  // the operator's plan (for callers that build on it)
    size_t KSpaceSize() const { return m_M; }
    size_t Maxit() const { return m_maxit; }
    RT Alpha() const { return m_alpha; }
    RT Epsilon() const { return m_epsilon; }

    virtual std::ostream &Print(std::ostream &os) const
    {
        Operator<T>::Print(os);
        os << "    image size: rank(" << Rank() << ") side(" << ImageSize() << ") nodes(" << KSpaceSize() << ")\n";
        os << "    nfft: maxit(" << m_maxit << ") eps(" << m_epsilon << ") alpha(" << m_alpha << ") m(" << m_m << ")\n";
        return os;
    }

private:
    size_t image_numel() const { size_t p = 1; for (size_t v : m_N) p *= v; return p; }
    // image dims of the adjoint: N.. plus the Cartesian stack (NFFT.hpp:378-379)
    std::vector<size_t> out_dims() const
    {
        std::vector<size_t> v = m_N;
        if (m_ncart > 1) v.push_back(m_ncart);
        return v;
    }
    void need_k() const { if (!m_have_k) throw std::logic_error("NFFT: k-space not set"); }

    void plan()
    {
        cgs_plan_desc d{};
        d.rank = (int)m_N.size();
        // codeare's first image index is the fastest; NFFT dimension 0 is the slowest
        for (int t = 0; t < d.rank; ++t) d.N[t] = (int)m_N[d.rank - 1 - t];
        d.alpha = m_alpha;
        d.m = (int)m_m;
        d.M = (int64_t)m_M;
        d.ncoils = (int)m_ncart;   // the slices of a Cartesian third dimension, else one
        cgs_host::check(cgs_plan_create(&m_plan, &d), "cgs_plan_create");
    }

    void release()
    {
        if (m_plan) cgs_plan_destroy(m_plan);
        m_plan = nullptr;
    }

    void steal(NFFT &o)
    {
        m_plan = o.m_plan; o.m_plan = nullptr;
        m_N = o.m_N; m_M = o.m_M; m_m = o.m_m; m_maxit = o.m_maxit; m_alpha = o.m_alpha;
        m_epsilon = o.m_epsilon; m_k = std::move(o.m_k); m_w = std::move(o.m_w); m_ncart = o.m_ncart;
        m_have_k = o.m_have_k; m_have_w = o.m_have_w;
    }

    cgs_plan *m_plan = nullptr;
    std::vector<size_t> m_N;
    size_t m_M = 0, m_m = 1, m_maxit = 3, m_ncart = 1;
    RT m_alpha = 1.f, m_epsilon = 7e-4f;
    Matrix<RT> m_k, m_w;
    bool m_have_k = false, m_have_w = false;
};
