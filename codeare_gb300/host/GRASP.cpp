// GRASP.cpp -- golden-angle radial sparse parallel reconstruction
// (GRASP.so), a drop-in for codeare's module of the same name (reference:
// src/modules/GRASP.cpp:31-230): stack-of-stars data sorted into contrast
// frames and reconstructed per slice by CS over NCSENSE with dim4 = frames.
//
// Defaults and keys are the reference's (GRASP.cpp:33-120): csiter 3,
// nliter 6, lsiter 6, cgmaxit 0 (the NCSENSE inverse is then codeare's E^H
// alone), tvw 0.02 (tvw1), tv (TV'ed axes), l1 1e-15, pnorm 1, nlopt 0, lsa
// 0.01, lsb 0.6, ftalpha 1, ftm 1, ftiter 1, fteps 7e-4,
// parallel_linesearch 1, ft 3, frame_duration 15, ta (acquisition time; the
// reference falls back to the workspace parameter "TA", which this
// workspace does not hold, so ta is required), margin_top, margin_bottom.
//   Process  meas (nx, nv, nz, nc), kspace (d, nx, nv), sensitivities
//            (N, N, nz, nc) -> im_xd (N, N, nz', nt): the slices inside the
//            margins, nt = ceil(ta / frame_duration) frames of
//            floor(nv / nt) views each, the density weights
//            linspace(1, 0.002, nx/2)^0.75, linspace(0.002, 1, nx/2)^0.75 per view
//            (GRASP.cpp:158-162), one CS_XSENSE per slice.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include "codeare/CS_XSENSE.hpp"
#include "codeare/ReconStrategy.hpp"

namespace RRStrategy {

class GRASP : public ReconStrategy {
public:
    GRASP() {}
    virtual ~GRASP() {}

    virtual codeare::error_code Init()
    {
        std::printf("Intialising GRASP ...\n");
        int i;
        float f;
        bool b;
        size_t z;
        if (Attribute("csiter", &i) == 0) m_csiter = i;
        if (Attribute("nliter", &i) == 0) m_nliter = i;
        if (Attribute("lsiter", &i) == 0) m_lsiter = i;
        if (Attribute("cgmaxit", &z) == 0) m_cgiter = z;
        if (Attribute("tvw", &f) == 0) m_tvw = f;
        if (Attribute("l1", &f) == 0) m_l1 = f;
        if (Attribute("pnorm", &f) == 0) m_pnorm = f;
        if (Attribute("verbose", &i) == 0) m_verbose = i;
        if (Attribute("nlopt", &i) == 0) m_nlopt = i;
        if (Attribute("lsa", &f) == 0) m_lsa = f;
        if (Attribute("lsb", &f) == 0) m_lsb = f;
        if (Attribute("ftalpha", &f) == 0) m_alpha = f;
        if (Attribute("ftm", &z) == 0) m_m = z;
        if (Attribute("ftiter", &i) == 0) m_ftiter = i;
        if (Attribute("fteps", &f) == 0) m_fteps = f;
        if (Attribute("parallel_linesearch", &b) == 0) m_pls = b;
        if (Attribute("ft", &i) == 0) m_ft = i;
        if (Attribute("frame_duration", &z) == 0) m_tf = z;
        std::string tv;
        if (Attribute("tv", &tv) == 0) {
            for (char &c : tv)
                if (c == ',') c = ' ';
            std::istringstream is(tv);
            size_t v;
            while (is >> v) m_tv.push_back(v);
        }
        if (Attribute("ta", &f) != 0) {
            std::printf("**ERROR - GRASP::Init: the acquisition time \"ta\" is required\n");
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        m_ta = f;
        if (Attribute("margin_top", &z) == 0) m_margin_top = z;
        if (Attribute("margin_bottom", &z) == 0) m_margin_bottom = z;
        if (m_ft != 3 || m_tf == 0 || !(m_ta > 0.f)) {
            std::printf("**ERROR - GRASP::Init: needs ft = 3, frame_duration > 0 and ta > 0\n");
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        std::printf("... done.\n\n");
        m_initialised = true;
        return codeare::OK;
    }

    virtual codeare::error_code Prepare() { return codeare::OK; }

    virtual codeare::error_code Process()
    {
        if (!m_initialised) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            const Matrix<cxfl> &meas = Get<cxfl>("meas");
            const Matrix<float> &kspace = Get<float>("kspace");
            const Matrix<cxfl> &sens = Get<cxfl>("sensitivities");
            const size_t nx = meas.Dim(0), NV = meas.Dim(1), nz0 = meas.Dim(2), nc = meas.Dim(3);
            const size_t d = kspace.Dim(0), N0 = sens.Dim(0), N1 = sens.Dim(1);
            if (m_margin_top + m_margin_bottom >= nz0 || sens.Dim(2) != nz0 || sens.Dim(3) != nc ||
                kspace.Dim(1) != nx || kspace.Dim(2) < NV || d != 2 || nx < 2 || (nx & 1)) {
                std::printf("**ERROR - GRASP::Process: meas (nx, nv, nz, nc), kspace (2, nx, nv) and "
                            "sensitivities (N, N, nz, nc) do not match\n");
                return codeare::UNSUPPORTED_DIMENSION;
            }
            const size_t nz = nz0 - m_margin_top - m_margin_bottom;
            const size_t nt = (size_t)std::ceil(m_ta / (float)m_tf);
            const size_t nv = NV / nt, M = nx * nv;
            if (nt < 1 || nv < 1) {
                std::printf("**ERROR - GRASP::Process: fewer views than frames\n");
                return codeare::UNSUPPORTED_DIMENSION;
            }
            std::printf("  Data acquired within %gs\n  Sorting data in %zu contrast gates with %zu views each.\n",
                        m_ta, nt, nv);
            // density weights (GRASP.cpp:158-162): float linspace ramps ^ 0.75, repeated per view
            std::vector<float> w(M);
            const std::vector<float> down = linspace(1.f, 0.002f, nx / 2), up = linspace(0.002f, 1.f, nx / 2);
            for (size_t i = 0; i < nx / 2; ++i) {
                w[i] = (float)std::pow((double)down[i], 0.75);
                w[nx / 2 + i] = (float)std::pow((double)up[i], 0.75);
            }
            for (size_t v = 1; v < nv; ++v)
                for (size_t i = 0; i < nx; ++i) w[v * nx + i] = w[i];
            Matrix<float> wm(M, 1);
            for (size_t j = 0; j < M; ++j) wm[j] = w[j];
            // the first nt * nv views, frame t = views [t nv, (t+1) nv): (d, nx nv, nt)
            Matrix<float> km(d, M, nt);
            for (size_t j = 0; j < d * M * nt; ++j) km[j] = kspace[j];
            Matrix<cxfl> im_xd(N0, N1, nz, nt);
            for (size_t iz = 0; iz < nz; ++iz) {
                const size_t z0 = iz + m_margin_top;
                Matrix<cxfl> sz(N0, N1, nc);
                for (size_t c = 0; c < nc; ++c)
                    for (size_t q = 0; q < N0 * N1; ++q) sz[q + N0 * N1 * c] = sens[q + N0 * N1 * (z0 + nz0 * c)];
                // (nx nv, nc, nt): sample j = ix + nx iv of view iv + nv t
                Matrix<cxfl> yz(M, nc, nt);
                for (size_t t = 0; t < nt; ++t)
                    for (size_t c = 0; c < nc; ++c)
                        for (size_t iv = 0; iv < nv; ++iv)
                            for (size_t ix = 0; ix < nx; ++ix)
                                yz[ix + nx * iv + M * (c + nc * t)] =
                                    meas[ix + nx * (iv + nv * t + NV * (z0 + nz0 * c))];
                Params p;
                p["sensitivities"] = sz;
                p["imsz"] = std::vector<size_t>{N0, N1};
                p["dim4"] = nt;
                p["nk"] = M;
                p["cgeps"] = 1.0e-6f;
                p["csiter"] = m_csiter;
                p["cgconv"] = 0.0f;
                p["lsiter"] = m_lsiter;
                p["xfmw"] = 0.0f;
                p["m"] = m_m;
                p["cgiter"] = m_cgiter;
                p["lambda"] = 1.0e-9f;
                p["tvw1"] = m_tvw;
                p["tv1"] = m_tv;
                p["l1"] = m_l1;
                p["pnorm"] = m_pnorm;
                p["lsa"] = m_lsa;
                p["nlopt"] = m_nlopt;
                p["lsb"] = m_lsb;
                p["alpha"] = m_alpha;
                p["fteps"] = m_fteps;
                p["parallel_linesearch"] = m_pls;
                p["ft"] = m_ft;
                p["ftiter"] = (size_t)m_ftiter;
                p["nliter"] = m_nliter;
                p["verbose"] = m_verbose;
                CS_XSENSE<cxfl> ft(p);
                ft.KSpace(km);
                ft.Weights(wm);
                const Matrix<cxfl> x = ft->*yz;
                for (size_t t = 0; t < nt; ++t)
                    for (size_t q = 0; q < N0 * N1; ++q) im_xd[q + N0 * N1 * (iz + nz * t)] = x[q + N0 * N1 * t];
                if (m_verbose) {
                    const cgs_cs_report &r = ft.LastReport();
                    std::printf("  slice %zu: %d NLCG iterations, %.3f s\n", iz, r.iterations, r.seconds);
                }
            }
            Add("im_xd", im_xd);
        } catch (const codeare::error_code &e) {
            return e;
        } catch (const std::exception &e) {
            std::printf("**ERROR - GRASP::Process: %s\n", e.what());
            return codeare::ERROR_GENERAL;
        }
        return codeare::OK;
    }

    virtual codeare::error_code Finalise() { return codeare::OK; }

private:
    // codeare's linspace: float steps accumulated from start, end set exactly
    // (src/matrix/Creators.hpp:573-590)
    static std::vector<float> linspace(float a, float b, size_t n)
    {
        std::vector<float> r(n, a);
        if (n < 2) return r;
        const float gap = (b - a) / (float)(n - 1);
        r[n - 1] = b;
        for (size_t i = 1; i + 1 < n; ++i) r[i] = r[i - 1] + gap;
        return r;
    }

    int m_csiter = 3, m_nliter = 6, m_lsiter = 6, m_verbose = 0, m_nlopt = 0, m_ftiter = 1, m_ft = 3;
    size_t m_cgiter = 0, m_m = 1, m_tf = 15, m_margin_top = 0, m_margin_bottom = 0;
    float m_tvw = 0.02f, m_l1 = 1.0e-15f, m_pnorm = 1.f, m_lsa = 0.01f, m_lsb = 0.6f, m_alpha = 1.f,
          m_fteps = 7.0e-4f, m_ta = 0.f;
    bool m_pls = true;
    std::vector<size_t> m_tv;
};

}  // namespace RRStrategy

extern "C" DLLEXPORT RRStrategy::ReconStrategy *create() { return new RRStrategy::GRASP; }
extern "C" DLLEXPORT void destroy(RRStrategy::ReconStrategy *p) { delete p; }
