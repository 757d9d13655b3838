// CGSENSE.cpp -- the CG-SENSE ReconStrategy plugin (CGSENSE.so), a drop-in
// for codeare's module of the same name (reference:
// src/modules/CGSENSE.hpp:25-105, src/modules/CGSENSE.cpp:52-191).
//
// Lifecycle and keys are the reference's:
//   Init     reads nk, lambda (default 5e-2), m, testcase, threads, verbose,
//            dft_3rd_dim, noise, cgeps, cgmaxit, ftmaxit, fteps
//   Prepare  builds the NCSENSE operator from "sensitivities", sets "kspace"
//            and "weights", then frees those two workspace entries
//   Process  image = NCSENSE ->* signals (or of the forward model of a
//            Shepp-Logan phantom in test-case mode, plus optional noise)
// As in the reference, the oversampling factor is not forwarded (sigma = 1)
// and fteps is read but not forwarded (the inner threshold stays 1e-3).
// Optional keys with no reference counterpart (defaults reproduce the
// reference): alpha (oversampling), mode ("codeare" | "standard"),
// weighted (standard mode), seed (test-case noise; the reference seeds from
// the clock, RandTraits.hpp:119-124).
#include <cstdio>
#include <random>
#include <string>

#include "codeare/CGLS.hpp"
#include "codeare/Creators.hpp"
#include "codeare/NCSENSE.hpp"
#include "codeare/ReconStrategy.hpp"

namespace RRStrategy {

class CGSENSE : public ReconStrategy {
public:
    CGSENSE() {}
    virtual ~CGSENSE() { Finalise(); }

    virtual codeare::error_code Init()
    {
        std::printf("Intialising CG-SENSE ...\n");
        m_initialised = false;
        m_testcase = 0;
        m_verbose = 0;
        m_noise = 0;
        m_lambda = 5.0e-2f;
        Attribute("nk", &m_nk);
        std::printf("  nk       : %i \n", m_nk);
        Attribute("lambda", &m_lambda);
        Attribute("m", &m_m);
        Attribute("testcase", &m_testcase);
        std::printf("  test case: %i \n", m_testcase);
        Attribute("threads", &m_nthreads);
        std::printf("  # of threads: %i \n", m_nthreads);
        Attribute("verbose", &m_verbose);
        std::printf("  verbose feedback: %i \n", m_verbose);
        Attribute("dft_3rd_dim", &m_3rd_dim_cart);
        std::printf("  Cartesian 3rd dimension: %d \n", m_3rd_dim_cart);
        Attribute("noise", &m_noise);
        std::printf("  gaussian white noise (normalised): %.9f \n", m_noise);
        Attribute("cgeps", &m_cgeps);
        Attribute("cgmaxit", &m_cgmaxit);
        std::printf("  maximum #iterations: %i \n", m_cgmaxit);
        std::printf("  convergence criterium: %.9f \n", m_cgeps);
        Attribute("ftmaxit", &m_ftmaxit);
        Attribute("fteps", &m_fteps);
        // keys without a reference counterpart (silent when absent)
        if (const char *a = Configurable::Attribute("alpha")) m_alpha = std::atof(a);
        if (const char *a = Configurable::Attribute("mode")) m_mode = a;
        if (const char *a = Configurable::Attribute("weighted")) m_weighted = std::atoi(a);
        if (const char *a = Configurable::Attribute("toeplitz")) m_toeplitz = std::atoi(a);
        if (const char *a = Configurable::Attribute("seed")) m_seed = (unsigned)std::atol(a);
        std::printf("... done.\n\n");
        return codeare::OK;
    }

    virtual codeare::error_code Prepare()
    {
        try {
            Params cgp;
            cgp["sensitivities"] = Get<cxfl>("sensitivities");
            cgp["nk"] = (size_t)m_nk;
            cgp["verbose"] = m_verbose;
            cgp["ftiter"] = (size_t)m_ftmaxit;
            cgp["cgiter"] = (size_t)m_cgmaxit;
            cgp["cgeps"] = m_cgeps;
            cgp["lambda"] = m_lambda;
            cgp["threads"] = m_nthreads;
            cgp["m"] = m_m;
            cgp["3rd_dim_cart"] = m_3rd_dim_cart;
            if (m_alpha != 1.0) cgp["alpha"] = m_alpha;
            cgp["mode"] = m_mode;
            cgp["weighted"] = m_weighted;
            cgp["toeplitz"] = m_toeplitz;
            m_ncs = NCSENSE<cxfl>(cgp);
            m_ncs.KSpace(Get<float>("kspace"));
            m_ncs.Weights(Get<float>("weights"));
        } catch (const std::exception &e) {
            std::printf("**ERROR - CGSENSE::Prepare: %s\n", e.what());
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        } catch (const codeare::error_code &e) {
            std::printf("**ERROR - CGSENSE::Prepare: missing workspace matrix\n");
            return e;
        } catch (...) {
            std::printf("**ERROR - CGSENSE::Prepare: bad k-space dimensions\n");
            return codeare::UNSUPPORTED_DIMENSION;
        }
        Free("weights");
        Free("kspace");
        std::printf("\n");
        m_initialised = true;
        return codeare::OK;
    }

    virtual codeare::error_code Process()
    {
        if (!m_initialised) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            const Matrix<cxfl> &sens = Get<cxfl>("sensitivities");
            Matrix<cxfl> data = (!m_testcase) ? Get<cxfl>("signals") : m_ncs.Trafo(phantom<cxfl>(size(sens, 0)));
            if (m_noise) {
                std::mt19937 gen(m_seed);
                std::normal_distribution<float> nd(0.f, 1.f);
                for (auto &v : data.Container()) v += m_noise * cxfl(nd(gen), nd(gen));
            }
            Matrix<cxfl> img = m_ncs->*data;
            Add("image", img);
        } catch (const std::exception &e) {
            std::printf("**ERROR - CGSENSE::Process: %s\n", e.what());
            return codeare::ERROR_GENERAL;
        } catch (const codeare::error_code &e) {
            return e;
        }
        return codeare::OK;
    }

    virtual codeare::error_code Finalise() { return codeare::OK; }

    const NCSENSE<cxfl> &Operator() const { return m_ncs; }

private:
    NCSENSE<cxfl> m_ncs;
    int m_verbose = 0, m_testcase = 0, m_ftmaxit = 3, m_cgmaxit = 10, m_nthreads = 0, m_nk = 1, m_m = 1;
    bool m_3rd_dim_cart = false;
    float m_noise = 0.f, m_lambda = 1.0e-6f, m_fteps = 1.0e-3f, m_cgeps = 1.0e-7f;
    double m_alpha = 1.0;
    std::string m_mode = "codeare";
    int m_weighted = 1, m_toeplitz = 0;
    unsigned m_seed = 0;
};

}  // namespace RRStrategy

extern "C" DLLEXPORT RRStrategy::ReconStrategy *create() { return new RRStrategy::CGSENSE; }
extern "C" DLLEXPORT void destroy(RRStrategy::ReconStrategy *p) { delete p; }
