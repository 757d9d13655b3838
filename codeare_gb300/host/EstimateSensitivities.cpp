// EstimateSensitivities.cpp -- coil-sensitivity estimation from golden-angle
// radial data (EstimateSensitivities.so), the step before CG-SENSE that
// produces its "sensitivities" input (reference:
// src/modules/EstimateSensitivities.cpp:53-182).
//
//   Init     reads ftalpha, ftm, nk, nl, cart_3rd_dim, image_size ("N0 N1"),
//            ftiter (CGNR steps of the inverse NFFT, default 3)
//   Prepare  takes the "sync" trajectory of one spoke on the gradient raster:
//            column 0 holds interleaved (kx, ky) pairs
//   Process  "meas" (nk x nc x nv complex, per volume one spoke) is scaled by
//            1e6; the spoke is interpolated linearly to ten times the raster
//            and cut to nk samples; volume v is that spoke rotated by v times
//            the golden angle; the nodes are scaled by 1 / (2 max |k|); all
//            coils are reconstructed together by the inverse NFFT (CGNR,
//            unit weights) on the GPU; "sensitivities" (N0 x N1 x nc) and
//            "kspace" (2 x nk nv) are added to the workspace.
//
// Differences from the reference, each because the reference's own code does
// not do what its comments say:
//   - every coil is reconstructed (the reference's loop stops after coil 0);
//   - the rotation of volume v is v * golden_angle degrees (key golden_angle,
//     default 111.246117975); the reference takes exp(v * 111.246) as the
//     angle in radians, which overflows single precision for v >= 1;
//   - nodes at +0.5 after the scaling wrap to -0.5, as the NFFT is periodic;
//   - optional key normalise=1 divides by the root sum of squares over coils
//     (the reference has that step commented out; the default 0 keeps it so).
#include <cmath>
#include <complex>
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "cgs.h"
#include "codeare/ReconStrategy.hpp"

namespace RRStrategy {

class EstimateSensitivities : public ReconStrategy {
public:
    virtual ~EstimateSensitivities() { Finalise(); }

    virtual codeare::error_code Finalise()
    {
        if (m_plan) cgs_plan_destroy(m_plan);
        m_plan = nullptr;
        return codeare::OK;
    }

    virtual codeare::error_code Init()
    {
        m_initialised = false;
        Attribute("ftalpha", &m_alpha);
        Attribute("ftm", &m_m);
        Attribute("nk", &m_nk);
        Attribute("nl", &m_nl);
        Attribute("cart_3rd_dim", &m_cart3);
        Attribute("ftiter", &m_ftiter);
        Attribute("golden_angle", &m_golden);
        Attribute("normalise", &m_normalise);
        std::string sz;
        Attribute("image_size", &sz);
        std::istringstream is(sz);
        size_t v;
        m_imsz.clear();
        while (is >> v) m_imsz.push_back(v);
        if (m_imsz.size() != 2 || m_nk < 1 || m_ftiter < 0 || m_m < 1) {
            std::printf("**ERROR - EstimateSensitivities::Init: needs image_size \"N0 N1\", nk >= 1, ftm >= 1\n");
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        if (m_cart3 || m_nl > 1) {
            std::printf("**ERROR - EstimateSensitivities::Init: 2-D radial data only (nl = 1)\n");
            return codeare::UNSUPPORTED_DIMENSION;
        }
        Matrix<cxfl> sensitivities;
        Add("sensitivities", sensitivities);
        m_initialised = true;
        return codeare::OK;
    }

    virtual codeare::error_code Prepare()
    {
        try {
            const Matrix<float> &sync = Get<float>("sync");
            const size_t n = sync.Dim(0) / 2;  // column 0: interleaved (kx, ky)
            if (n < 2) return codeare::CONTEXT_CONFIGURATION_FAILED;
            m_raster.assign(2 * n, 0.f);
            for (size_t i = 0; i < 2 * n; ++i) m_raster[i] = sync.Ptr()[i];
        } catch (const codeare::error_code &e) {
            return e;
        }
        return codeare::OK;
    }

    virtual codeare::error_code Process()
    {
        if (!m_initialised) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            Matrix<cxfl> &meas = Get<cxfl>("meas");
            const size_t nk = meas.Dim(0), nc = meas.Dim(1), nv = meas.Dim(2) * meas.Dim(3);
            if (nk != (size_t)m_nk) {
                std::printf("**ERROR - EstimateSensitivities::Process: meas has %zu samples per spoke, nk = %d\n",
                            nk, m_nk);
                return codeare::CONTEXT_CONFIGURATION_FAILED;
            }
            const std::vector<float> kxy = trajectory(nk, nv);
            const size_t M = nk * nv;
            // samples per coil in trajectory order (sample fastest, then volume)
            std::vector<cxfl> y(M * nc);
            for (size_t v = 0; v < nv; ++v)
                for (size_t c = 0; c < nc; ++c)
                    for (size_t k = 0; k < nk; ++k)
                        y[c * M + v * nk + k] = meas.Ptr()[(v * nc + c) * nk + k] * 1e6f;
            cgs_plan_desc d{};
            d.rank = 2;
            d.N[0] = (int)m_imsz[1];  // slow image axis: codeare's second index
            d.N[1] = (int)m_imsz[0];
            d.N[2] = 1;
            d.alpha = m_alpha;
            d.m = m_m;
            d.M = (int64_t)M;
            d.ncoils = (int)nc;
            if (m_plan) cgs_plan_destroy(m_plan);
            m_plan = nullptr;
            std::vector<float> w(M, 1.f);
            Matrix<cxfl> sens(m_imsz[0], m_imsz[1], nc);
            if (cgs_plan_create(&m_plan, &d) != CGS_OK || cgs_set_kspace(m_plan, kxy.data()) != CGS_OK ||
                cgs_set_weights(m_plan, w.data()) != CGS_OK ||
                cgs_nfft_itrafo(m_plan, reinterpret_cast<const float *>(y.data()),
                                reinterpret_cast<float *>(sens.Ptr()), m_ftiter, 7e-4, nullptr) != CGS_OK) {
                std::printf("**ERROR - EstimateSensitivities::Process: %s\n", cgs_last_error());
                return codeare::ERROR_GENERAL;
            }
            if (m_normalise) normalise(sens, nc);
            Matrix<float> kspace(2, M);
            for (size_t i = 0; i < 2 * M; ++i) kspace.Ptr()[i] = kxy[i];
            Add("sensitivities", sens);
            Add("kspace", kspace);
        } catch (const codeare::error_code &e) {
            return e;
        } catch (const std::exception &e) {
            std::printf("**ERROR - EstimateSensitivities::Process: %s\n", e.what());
            return codeare::ERROR_GENERAL;
        }
        return codeare::OK;
    }

private:
    // (2, nk nv) nodes: the raster spoke linearly interpolated to 10x the
    // samples and cut to nk, rotated by v golden angles, scaled to |k| <= 1/2
    std::vector<float> trajectory(size_t nk, size_t nv) const
    {
        const size_t n = m_raster.size() / 2, nf = 10 * n;
        std::vector<std::complex<double>> spoke(nk);
        for (size_t j = 0; j < nk; ++j) {
            // XI = linspace(0, 1, nf) sampled against xi = linspace(0, 1, n)
            const double X = (nf > 1) ? (double)j / (double)(nf - 1) : 0.0;
            const double pos = X * (double)(n - 1);
            size_t i0 = (size_t)std::floor(pos);
            if (i0 >= n - 1) i0 = n - 2;
            const double f = pos - (double)i0;
            const double kx = (1 - f) * m_raster[2 * i0] + f * m_raster[2 * i0 + 2];
            const double ky = (1 - f) * m_raster[2 * i0 + 1] + f * m_raster[2 * i0 + 3];
            spoke[j] = std::complex<double>(kx, ky);
        }
        std::vector<std::complex<double>> k(nk * nv);
        double kmax = 0.0;
        for (size_t v = 0; v < nv; ++v) {
            const std::complex<double> rot = std::polar(1.0, (double)v * m_golden * M_PI / 180.0);
            for (size_t j = 0; j < nk; ++j) {
                k[v * nk + j] = spoke[j] * rot;
                kmax = std::max(kmax, std::abs(k[v * nk + j]));
            }
        }
        std::vector<float> out(2 * nk * nv);
        const double s = kmax > 0 ? 1.0 / (2.0 * kmax) : 1.0;
        auto wrap = [](double x) { return (float)(x >= 0.5 ? x - 1.0 : x); };
        for (size_t i = 0; i < nk * nv; ++i) {
            out[2 * i] = wrap(k[i].real() * s);
            out[2 * i + 1] = wrap(k[i].imag() * s);
        }
        return out;
    }

    static void normalise(Matrix<cxfl> &sens, size_t nc)
    {
        const size_t P = sens.Size() / nc;
        for (size_t p = 0; p < P; ++p) {
            double ss = 0.0;
            for (size_t c = 0; c < nc; ++c) ss += std::norm(sens.Ptr()[c * P + p]);
            const float inv = ss > 0.0 ? (float)(1.0 / std::sqrt(ss)) : 0.f;
            for (size_t c = 0; c < nc; ++c) sens.Ptr()[c * P + p] *= inv;
        }
    }

    cgs_plan *m_plan = nullptr;
    float m_alpha = 1.f;
    int m_m = 1, m_nk = 0, m_nl = 1, m_ftiter = 3;
    bool m_cart3 = false;
    int m_normalise = 0;
    double m_golden = 111.246117975;
    std::vector<size_t> m_imsz;
    std::vector<float> m_raster;
};

}  // namespace RRStrategy

extern "C" DLLEXPORT RRStrategy::ReconStrategy *create() { return new RRStrategy::EstimateSensitivities; }
extern "C" DLLEXPORT void destroy(RRStrategy::ReconStrategy *p) { delete p; }
