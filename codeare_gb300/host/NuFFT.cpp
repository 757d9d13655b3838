// NuFFT.cpp -- the single-channel non-Cartesian FT module (NuFFT.so), a
// drop-in for codeare's module of the same name (reference:
// src/modules/NuFFT.hpp, src/modules/NuFFT.cpp:50-146).
//
//   Init     reads dim, nx/ny/nz, M, shots, maxit, epsilon, dft_3rd_dim,
//            test_case, m (default 1), alpha (default 1) and builds an NFFT
//            with nk = M * shots; like the reference it does not forward
//            maxit and epsilon, so the inverse NFFT keeps 3 steps and 7e-4
//   Prepare  sets "kspace" and "weights", then frees them
//   Process  img = NFFT ->* data (the CGNR inverse NFFT), or of the forward
//            model of a Shepp-Logan phantom in test-case mode (2-D)
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "codeare/Creators.hpp"
#include "codeare/NFFT.hpp"
#include "codeare/ReconStrategy.hpp"

namespace RRStrategy {

class NuFFT : public ReconStrategy {
public:
    virtual ~NuFFT() { Finalise(); }

    virtual codeare::error_code Init()
    {
        m_initialised = false;
        int shots = 1, M = 1, maxit = 3, m = 1, N[4] = {1, 1, 1, 1};
        float epsilon = 7e-4f, alpha = 1.0f;
        const char *sides[3] = {"nx", "ny", "nz"};
        int dim = 2;
        Attribute("dim", &dim);
        if (dim < 2 || dim > 3) return codeare::UNSUPPORTED_DIMENSION;
        m_dim = (size_t)dim;
        for (int i = 0; i < dim; ++i) Attribute(sides[i], &N[i]);
        Attribute("M", &M);
        Attribute("shots", &shots);
        Attribute("maxit", &maxit);
        Attribute("epsilon", &epsilon);
        Attribute("dft_3rd_dim", &m_dft_3rd_dim);
        Attribute("test_case", &m_test_case);
        Attribute("m", &m);
        Attribute("alpha", &alpha);
        std::vector<size_t> ms(m_dim, 1);
        for (size_t i = 0; i < m_dim; ++i) ms[i] = (size_t)N[i];
        try {
            Params p;
            p["alpha"] = alpha;
            p["m"] = m;
            if (Exists<float>("b0") == codeare::OK) p["b0"] = Get<float>("b0");
            p["nk"] = M * shots;
            p["3rd_dim_cart"] = m_dft_3rd_dim;
            p["imsz"] = ms;
            ft = NFFT<cxfl>(p);
        } catch (const std::exception &e) {
            std::printf("**ERROR - NuFFT::Init: %s\n", e.what());
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        m_initialised = true;
        return codeare::OK;
    }

    virtual codeare::error_code Prepare()
    {
        try {
            ft.KSpace(Get<float>("kspace"));
            ft.Weights(Get<float>("weights"));
        } catch (const std::exception &e) {
            std::printf("**ERROR - NuFFT::Prepare: %s\n", e.what());
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        } catch (const codeare::error_code &e) {
            return e;
        }
        ft.Print(std::cout);
        Free("kspace");
        Free("weights");
        return codeare::OK;
    }

    virtual codeare::error_code Process()
    {
        if (!m_initialised) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            Matrix<cxfl> data;
            if (m_test_case) {
                if (m_dim != 2) return codeare::UNSUPPORTED_DIMENSION;
                data = ft * phantom<cxfl>(ft.ImageSize());
            } else {
                data = Get<cxfl>("data");
            }
            Matrix<cxfl> img = ft->*data;
            Add("img", img);
        } catch (const std::exception &e) {
            std::printf("**ERROR - NuFFT::Process: %s\n", e.what());
            return codeare::ERROR_GENERAL;
        } catch (const codeare::error_code &e) {
            return e;
        }
        return codeare::OK;
    }

private:
    NFFT<cxfl> ft;
    bool m_dft_3rd_dim = false;
    bool m_test_case = false;
    size_t m_dim = 2;
};

}  // namespace RRStrategy

extern "C" DLLEXPORT RRStrategy::ReconStrategy *create() { return new RRStrategy::NuFFT; }
extern "C" DLLEXPORT void destroy(RRStrategy::ReconStrategy *p) { delete p; }
