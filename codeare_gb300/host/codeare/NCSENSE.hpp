// NCSENSE.hpp -- GB300 non-Cartesian SENSE operator with the interface of
// codeare's NCSENSE<T> (reference: src/matrix/ft/NCSENSE.hpp:47-493).
//
// Params keys and defaults as the reference constructor (NCSENSE.hpp:69-184):
// sensitivities (required, (N.., NC)), nk, ftiter = 3, fteps = 1e-3,
// alpha = 1, m = 1, cgiter = 0, cgeps = 1e-6, lambda = 1e-6, verbose.  New
// optional keys: "mode" ("codeare" = the reference's CGLS over its CGNR-based
// E^H, the default; "standard" = CG on E^H W E + lambda with the true adjoint)
// "weighted" (standard mode: use the density weights, default 1) and
// "toeplitz" (1: every CG step's normal operator through the Toeplitz kernel
// of the trajectory; codeare mode then runs its inner CGNR in image space and
// needs alpha >= 2 and m >= 4; default 0).
//
//   Trafo / operator*   E: y_c = NFFT(S_c . x)            (NCSENSE.hpp:310-348)
//   operator/           codeare's E^H (mode codeare) or E^H W (standard)
//                                                          (NCSENSE.hpp:251-301)
//   Adjoint / ->*       the full CG-SENSE solve            (NCSENSE.hpp:408-436)
//
// dim4 / dim5 (NCSENSE.hpp:141-166, 204-348): dim4 x dim5 frames, each with
// its own trajectory (k-space (d, nk, dim4[, dim5])) and the shared
// sensitivities and weights; images (N.., dim4[, dim5]), signals
// (nk, NC, dim4[, dim5]); the CG-SENSE solve runs over the stacked frames.
// The whole solve runs on the GPU (libcgs.so cgs_solve); unlike the
// reference's CGLS member, no residual history survives between solves.
// 3rd_dim_cart (NCSENSE.hpp:81-97, 105; NFFT.hpp:100-103): sensitivities
// (N0, N1, slices, NC), images (N0, N1, slices), signals (nk, slices, NC);
// every slice is a 2-D problem with the shared trajectory and its own slice of
// the maps (a frame of the plan), and the CG-SENSE solve runs over the whole
// stack, as the reference's CGLS does over its (N0, N1, slices) images.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "NFFT.hpp"

enum FT_EXCEPTION { NCSENSE_KSPACE_DIMENSIONS };

template <class T> class NCSENSE : public FT<T> {
    typedef typename TypeTraits<T>::RT RT;

public:
    NCSENSE() {}

    explicit NCSENSE(const Params &params) : FT<T>(params)
    {
        if (!params.exists("sensitivities")) throw std::invalid_argument("NCSENSE: sensitivities required");
        m_sm = params.Get<Matrix<T>>("sensitivities");
        m_ftiter = params.exists("ftiter") ? unsigned_cast(params["ftiter"]) : 3;
        m_fteps = params.exists("fteps") ? fp_cast(params["fteps"]) : 1.0e-3;
        m_alpha = params.exists("alpha") ? fp_cast(params["alpha"]) : 1.0;
        m_m = params.exists("m") ? unsigned_cast(params["m"]) : 1;
        m_nk = params.exists("nk") ? unsigned_cast(params["nk"]) : 1;
        try { m_cgiter = params.Get<size_t>("cgiter"); } catch (...) {}
        try { m_cgeps = params.Get<RT>("cgeps"); } catch (...) {}
        try { m_lambda = params.Get<RT>("lambda"); } catch (...) {}
        try { m_verbose = params.Get<int>("verbose") > 0; } catch (...) {}
        if (params.exists("mode")) {
            const std::string md = params.Get<std::string>("mode");
            if (md == "standard") m_mode = CGS_MODE_STANDARD;
            else if (md == "codeare") m_mode = CGS_MODE_CODEARE;
            else throw std::invalid_argument("NCSENSE: mode must be codeare or standard");
        }
        m_weighted = try_to_fetch<int>(params, "weighted", 1);
        m_toeplitz = try_to_fetch<int>(params, "toeplitz", 0);
        m_cart = try_to_fetch<bool>(params, "3rd_dim_cart", false);
        m_dim4 = std::max<size_t>(1, try_to_fetch<size_t>(params, "dim4", 1));
        m_dim5 = std::max<size_t>(1, try_to_fetch<size_t>(params, "dim5", 1));
        if (m_cart && (m_dim4 > 1 || m_dim5 > 1))
            throw std::invalid_argument("NCSENSE: 3rd_dim_cart with dim4 / dim5 frames is not supported");
        plan();
    }

    NCSENSE(const NCSENSE &o) : FT<T>(o) { *this = o; }

    NCSENSE &operator=(const NCSENSE &o)
    {
        if (this == &o) return *this;
        release();
        this->m_params = o.m_params;
        m_sm = o.m_sm; m_k = o.m_k; m_w = o.m_w;
        m_ftiter = o.m_ftiter; m_fteps = o.m_fteps; m_alpha = o.m_alpha; m_m = o.m_m; m_nk = o.m_nk;
        m_dim4 = o.m_dim4; m_dim5 = o.m_dim5; m_cart = o.m_cart;
        m_cgiter = o.m_cgiter; m_cgeps = o.m_cgeps; m_lambda = o.m_lambda; m_verbose = o.m_verbose;
        m_mode = o.m_mode; m_weighted = o.m_weighted; m_toeplitz = o.m_toeplitz; m_have_k = o.m_have_k;
        m_have_w = o.m_have_w;
        if (o.m_plan) {
            plan();
            if (m_have_k) KSpace(m_k);
            if (m_have_w) Weights(m_w);
        }
        return *this;
    }

    NCSENSE(NCSENSE &&o) noexcept : FT<T>(o) { steal(o); }
    NCSENSE &operator=(NCSENSE &&o) noexcept
    {
        if (this != &o) { release(); this->m_params = o.m_params; steal(o); }
        return *this;
    }

    virtual ~NCSENSE() { release(); }

    virtual void Sensitivities(const Matrix<T> &sm)
    {
        if (sm.Size() != m_sm.Size()) throw std::invalid_argument("NCSENSE: sensitivity size changed");
        m_sm = sm;
        set_maps();
    }

    virtual void KSpace(const Matrix<RT> &k)
    {
        if (m_cart) {
            // one trajectory for every slice (the reference broadcasts it to
            // each coil's NFFT, NCSENSE.hpp:204-223): one copy per frame
            if (size(k, 1) != m_nk || size(k, 0) != m_rank || k.Size() != m_rank * m_nk)
                throw NCSENSE_KSPACE_DIMENSIONS;
            m_k = k;
            Matrix<RT> kk(m_rank, m_nk, m_ncart);
            for (size_t z = 0; z < m_ncart; ++z)
                std::copy(k.Ptr(), k.Ptr() + k.Size(), kk.Ptr() + z * k.Size());
            cgs_host::check(cgs_set_kspace(m_plan, kk.Ptr()), "cgs_set_kspace");
            m_have_k = true;
            if (m_have_w) cgs_host::check(cgs_set_weights(m_plan, m_w.Ptr()), "cgs_set_weights");
            return;
        }
        if (size(k, 1) != m_nk || size(k, 0) != m_rank || k.Size() != m_rank * m_nk * frames())
            throw NCSENSE_KSPACE_DIMENSIONS;
        m_k = k;
        cgs_host::check(cgs_set_kspace(m_plan, k.Ptr()), "cgs_set_kspace");
        m_have_k = true;
        if (m_have_w) cgs_host::check(cgs_set_weights(m_plan, m_w.Ptr()), "cgs_set_weights");
    }

    virtual void Weights(const Matrix<RT> &w)
    {
        if (w.Size() != m_nk) throw std::invalid_argument("NCSENSE: weights must hold nk values");
        m_w = w;
        m_have_w = true;
        if (m_have_k) cgs_host::check(cgs_set_weights(m_plan, w.Ptr()), "cgs_set_weights");
    }

    virtual Matrix<T> Trafo(const MatrixType<T> &m) const
    {
        if (m_cart) {
            // the plan writes (nk, NC, slice); the reference's m_fwd_out is
            // (nk, slice, NC) (NCSENSE.hpp:105)
            Matrix<T> tmp(m_nk, m_nc, m_ncart);
            cgs_host::check(cgs_sense_trafo(m_plan, reinterpret_cast<const float *>(m.Ptr()),
                                            reinterpret_cast<float *>(tmp.Ptr()), nullptr), "cgs_sense_trafo");
            return cart_swap(tmp, m_nc, m_ncart);
        }
        std::vector<size_t> od{m_nk, m_nc};  // m_fwd_out (NCSENSE.hpp:173)
        if (frames() > 1) od.push_back(m_dim4);
        if (m_dim5 > 1) od.push_back(m_dim5);
        Matrix<T> out(od);
        cgs_host::check(cgs_sense_trafo(m_plan, reinterpret_cast<const float *>(m.Ptr()),
                                        reinterpret_cast<float *>(out.Ptr()), nullptr), "cgs_sense_trafo");
        return squeeze(out);
    }
    virtual Matrix<T> Trafo(const MatrixType<T> &m, const MatrixType<T> &, const bool & = true) const { return Trafo(m); }

    virtual Matrix<T> operator/(const MatrixType<T> &m) const
    {
        const Matrix<T> mc = m_cart ? plan_order(m) : Matrix<T>();
        const MatrixType<T> &in = m_cart ? mc : m;
        Matrix<T> out(image_dims());
        if (m_mode == CGS_MODE_CODEARE)
            cgs_host::check(cgs_sense_adjoint_codeare(m_plan, reinterpret_cast<const float *>(in.Ptr()),
                                                      reinterpret_cast<float *>(out.Ptr()), (int)m_ftiter,
                                                      (double)m_fteps, nullptr), "cgs_sense_adjoint_codeare");
        else
            cgs_host::check(cgs_sense_adjoint(m_plan, reinterpret_cast<const float *>(in.Ptr()),
                                              reinterpret_cast<float *>(out.Ptr()), m_weighted, nullptr),
                            "cgs_sense_adjoint");
        return out;
    }

    virtual Matrix<T> Adjoint(const MatrixType<T> &m) const
    {
        const Matrix<T> mc = m_cart ? plan_order(m) : Matrix<T>();
        const MatrixType<T> &in = m_cart ? mc : m;
        Matrix<T> out(image_dims());
        cgs_solve_opts o{};
        o.mode = m_mode; o.cgiter = (int)m_cgiter; o.cgeps = m_cgeps; o.lambda = m_lambda;
        o.ftiter = (int)m_ftiter; o.fteps = m_fteps; o.weighted = m_weighted; o.toeplitz = m_toeplitz;
        cgs_solve_report r{};
        cgs_status s = cgs_solve(m_plan, reinterpret_cast<const float *>(in.Ptr()), reinterpret_cast<float *>(out.Ptr()),
                                 &o, &r, nullptr);
        if (s != CGS_OK && s != CGS_ERR_NAN) cgs_host::check(s, "cgs_solve");
        m_last = r;
        // the reference prints the residual at which it stopped (CGLS.hpp:42-46)
        const int last = r.iterations < 256 ? r.iterations : 255;
        if (m_verbose)
            for (int i = 0; i <= last && i < 256; ++i) std::printf("    %03d %.7f\n", i, r.res_hist[i]);
        return out;
    }
    virtual Matrix<T> Adjoint(const MatrixType<T> &m, const MatrixType<T> &, const bool = false) const { return Adjoint(m); }

    virtual Matrix<T> operator*(const MatrixType<T> &m) const { return Trafo(m); }
    virtual Matrix<T> operator->*(const MatrixType<T> &m) const { return Adjoint(m); }

    size_t KSpaceSize() const { return m_nk; }
    size_t frames() const { return m_cart ? m_ncart : m_dim4 * m_dim5; }
    // image dims: N.. plus dim4 (and dim5) when batched (m_bwd_out without NC, NCSENSE.hpp:175-180);
    // with a Cartesian third dimension N0, N1 and the slices
    std::vector<size_t> image_dims() const
    {
        std::vector<size_t> v = m_imsz;
        if (m_cart) { v.push_back(m_ncart); return v; }
        if (frames() > 1) v.push_back(m_dim4);
        if (m_dim5 > 1) v.push_back(m_dim5);
        return v;
    }
    const std::vector<size_t> &ImageSize() const { return m_imsz; }
    cgs_plan *Plan() const { return m_plan; }  // the operator's plan (for callers that build on it)
    const cgs_solve_report &LastReport() const { return m_last; }

    virtual std::ostream &Print(std::ostream &os) const
    {
        Operator<T>::Print(os);
        os << "    NCCG: eps(" << m_cgeps << ") iter(" << m_cgiter << ") lambda(" << m_lambda << ")\n";
        os << "    channels(" << m_nc << ") mode(" << (m_mode == CGS_MODE_CODEARE ? "codeare" : "standard") << ")\n";
        return os;
    }

private:
    void plan()
    {
        const size_t nd = ndims(m_sm);
        if (nd < 3 || nd > 4) throw std::invalid_argument("NCSENSE: sensitivities must be (N,N[,N],NC)");
        m_rank = nd - 1;
        m_nc = size(m_sm, nd - 1);
        if (m_cart) {
            // (N0, N1, slices, NC): 2-D NFFTs per slice (NCSENSE.hpp:89-90)
            if (nd != 4) throw std::invalid_argument("NCSENSE: 3rd_dim_cart needs sensitivities (N,N,slices,NC)");
            m_rank = 2;
            m_ncart = size(m_sm, 2);
        }
        m_imsz.assign(m_rank, 0);
        for (size_t i = 0; i < m_rank; ++i) m_imsz[i] = size(m_sm, i);
        cgs_plan_desc d{};
        d.rank = (int)m_rank;
        for (size_t t = 0; t < m_rank; ++t) d.N[t] = (int)m_imsz[m_rank - 1 - t];
        d.alpha = m_alpha;
        d.m = (int)m_m;
        d.M = (int64_t)m_nk;
        d.ncoils = (int)m_nc;
        d.frames = (int)frames();
        cgs_host::check(cgs_plan_create(&m_plan, &d), "cgs_plan_create");
        set_maps();
    }

    void set_maps()
    {
        if (!m_cart) {
            cgs_host::check(cgs_set_sensitivities(m_plan, reinterpret_cast<const float *>(m_sm.Ptr())),
                            "cgs_set_sensitivities");
            return;
        }
        // slice z of every coil: (N0 N1) values at (c * slices + z) * N0 N1
        const size_t px = m_imsz[0] * m_imsz[1];
        Matrix<T> sl(m_imsz[0], m_imsz[1], m_nc);
        for (size_t z = 0; z < m_ncart; ++z) {
            for (size_t c = 0; c < m_nc; ++c)
                std::copy(m_sm.Ptr() + (c * m_ncart + z) * px, m_sm.Ptr() + (c * m_ncart + z + 1) * px,
                          sl.Ptr() + c * px);
            cgs_host::check(cgs_set_frame_sensitivities(m_plan, (int)z, reinterpret_cast<const float *>(sl.Ptr())),
                            "cgs_set_frame_sensitivities");
        }
    }

    // (a, b, nk) <-> (b, a, nk) in codeare order: swaps the slice and coil axes of signals
    static Matrix<T> cart_swap(const Matrix<T> &in, size_t a, size_t b)
    {
        const size_t nk = size(in, 0);
        Matrix<T> out(nk, b, a);
        for (size_t i = 0; i < a; ++i)
            for (size_t j = 0; j < b; ++j)
                std::copy(in.Ptr() + (j * a + i) * nk, in.Ptr() + (j * a + i + 1) * nk, out.Ptr() + (i * b + j) * nk);
        return out;
    }

    // the caller's signals (nk, slices, NC) in the plan's order (nk, NC, slices)
    Matrix<T> plan_order(const MatrixType<T> &m) const
    {
        if (m.Size() != m_nk * m_ncart * m_nc) throw std::invalid_argument("NCSENSE: signals must be (nk, slices, NC)");
        Matrix<T> in(m_nk, m_ncart, m_nc);
        std::copy(m.Ptr(), m.Ptr() + m.Size(), in.Ptr());
        return cart_swap(in, m_ncart, m_nc);
    }

    void release()
    {
        if (m_plan) cgs_plan_destroy(m_plan);
        m_plan = nullptr;
    }

    void steal(NCSENSE &o)
    {
        m_plan = o.m_plan; o.m_plan = nullptr;
        m_sm = std::move(o.m_sm); m_k = std::move(o.m_k); m_w = std::move(o.m_w); m_imsz = o.m_imsz;
        m_rank = o.m_rank; m_nc = o.m_nc; m_nk = o.m_nk; m_ftiter = o.m_ftiter; m_m = o.m_m;
        m_dim4 = o.m_dim4; m_dim5 = o.m_dim5; m_cart = o.m_cart; m_ncart = o.m_ncart;
        m_cgiter = o.m_cgiter; m_fteps = o.m_fteps; m_alpha = o.m_alpha; m_cgeps = o.m_cgeps;
        m_lambda = o.m_lambda; m_verbose = o.m_verbose; m_have_k = o.m_have_k; m_have_w = o.m_have_w;
        m_mode = o.m_mode; m_weighted = o.m_weighted; m_toeplitz = o.m_toeplitz; m_last = o.m_last;
    }

    cgs_plan *m_plan = nullptr;
    Matrix<T> m_sm;
    Matrix<RT> m_k, m_w;
    std::vector<size_t> m_imsz;
    size_t m_rank = 2, m_nc = 1, m_nk = 1, m_ftiter = 3, m_m = 1, m_cgiter = 0, m_dim4 = 1, m_dim5 = 1, m_ncart = 1;
    bool m_cart = false;
    double m_fteps = 1e-3, m_alpha = 1.0;
    RT m_cgeps = 1.0e-6f, m_lambda = 1.0e-6f;
    bool m_verbose = false, m_have_k = false, m_have_w = false;
    int m_mode = CGS_MODE_CODEARE, m_weighted = 1, m_toeplitz = 0;
    mutable cgs_solve_report m_last{};
};
