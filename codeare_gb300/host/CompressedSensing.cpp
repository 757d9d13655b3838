// CompressedSensing.cpp -- the compressed-sensing ReconStrategy plugin
// (CompressedSensing.so), a drop-in for codeare's module of the same name
// with ft = 3 (CS over the non-Cartesian SENSE operator) and ft = 2 (CS over
// the plain NFFT) (reference: src/modules/CompressedSensing.cpp:31-205).
//
// Lifecycle, keys and workspace names are the reference's:
//   Init     ftdims ("N0 N1 [N2]"), test_case, noise, ft, verbose; for
//            ft = 3 the NCSENSE keys nk, ftmaxit, fteps, cgmaxit, cgeps,
//            lambda, cart_3rd_dim, ftalpha (workspace "sensitivities"); for
//            ft = 2 the NFFT keys fteps, ftalpha, ftiter, ftm, ftnk; then
//            the CS keys nlopt, parallel_linesearch, tvw1, tvw2, tv1, xfmw,
//            l1, lsa, lsb, pnorm, wl_family, wl_member, csiter, cgiter (the
//            NLCG iterations), cgconv, lsiter
//   Prepare  sets "kspace" and "weights" on the operator, frees both
//   Process  im_dc = CS_XSENSE ->* data ("data", or the forward model of a
//            Shepp-Logan phantom when test_case is set, plus optional noise)
// The reference reads every key with RHSAttribute, whose value is undefined
// when the key is absent; here absent keys take CS_XSENSE's own defaults
// (zero weights and iterations, wl_family -1).  ft = 0 and 1 (Cartesian) are
// not served; test_case needs a 2-D image (the 3-D phantom is not provided);
// an optional key seed fixes the noise (the reference seeds from the clock).
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "codeare/CS_XSENSE.hpp"
#include "codeare/Creators.hpp"
#include "codeare/ReconStrategy.hpp"

namespace RRStrategy {

class CompressedSensing : public ReconStrategy {
public:
    CompressedSensing() {}
    virtual ~CompressedSensing() { Finalise(); }

    virtual codeare::error_code Init()
    {
        std::printf("Intialising CompressedSensing ...\n");
        m_initialised = false;
        Attribute("verbose", &m_verbose);
        m_image_size = list("ftdims");
        m_dim = m_image_size.size();
        if (m_dim < 2 || m_dim > 3) {
            std::printf("**ERROR - CompressedSensing::Init: ftdims must hold 2 or 3 sizes\n");
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        std::printf("  Geometry: %zuD (%zu,%zu,%zu)\n", m_dim, m_image_size[0], m_image_size[1],
                    m_dim == 3 ? m_image_size[2] : (size_t)1);
        Attribute("test_case", &m_test_case);
        Attribute("noise", &m_noise);
        Attribute("ft", &m_ft_type);
        if (m_ft_type != 3 && m_ft_type != 2) {
            std::printf("**ERROR - CompressedSensing::Init: ft = %d; this module serves ft = 2 (NFFT) and 3 "
                        "(NCSENSE)\n", m_ft_type);
            return codeare::UNSUPPORTED_DIMENSION;
        }
        if (m_test_case && m_dim != 2) {
            std::printf("**ERROR - CompressedSensing::Init: test_case needs a 2-D image\n");
            return codeare::UNSUPPORTED_DIMENSION;
        }
        std::printf("  FFT class: %s\n", m_ft_type == 3 ? "NCSENSE" : "NUFFT");
        try {
            Params p;
            int i = 0; float f = 0.f; bool b = false;
            if (m_ft_type == 3) {  // CompressedSensing.cpp:86-101
                p["sensitivities"] = Get<cxfl>("sensitivities");
                if (Attribute("nk", &i) == 0) p["nk"] = (size_t)i;
                if (Attribute("ftmaxit", &i) == 0) p["ftiter"] = (size_t)i;
                if (Attribute("fteps", &f) == 0) p["fteps"] = f;
                if (Attribute("cgmaxit", &i) == 0) p["cgiter"] = (size_t)i;
                if (Attribute("cgeps", &f) == 0) p["cgeps"] = f;
                if (Attribute("lambda", &f) == 0) p["lambda"] = f;
            } else {  // CompressedSensing.cpp:73-85
                if (Attribute("fteps", &f) == 0) p["epsilon"] = f;
                if (Attribute("ftiter", &i) == 0) p["maxit"] = (size_t)i;
                if (Attribute("ftm", &i) == 0) p["m"] = (size_t)i;
                if (Attribute("ftnk", &i) == 0) p["nk"] = (size_t)i;
            }
            if (Attribute("cart_3rd_dim", &b) == 0) p["3rd_dim_cart"] = b;
            if (Attribute("ftalpha", &f) == 0) p["alpha"] = f;
            p["imsz"] = m_image_size;
            if (Attribute("nlopt", &i) == 0) p["nlopt"] = i;
            if (Attribute("parallel_linesearch", &b) == 0) p["parallel_linesearch"] = b;
            if (Attribute("tvw1", &f) == 0) p["tvw1"] = f;
            if (Attribute("tvw2", &f) == 0) p["tvw2"] = f;
            p["tv1"] = list("tv1");
            if (Attribute("xfmw", &f) == 0) p["xfmw"] = f;
            if (Attribute("l1", &f) == 0) p["l1"] = f;
            if (Attribute("lsa", &f) == 0) p["lsa"] = f;
            if (Attribute("lsb", &f) == 0) p["lsb"] = f;
            if (Attribute("pnorm", &f) == 0) p["pnorm"] = f;
            p["verbose"] = m_verbose;
            if (Attribute("wl_family", &i) == 0) p["wl_family"] = i;
            if (Attribute("wl_member", &i) == 0) p["wl_member"] = i;
            if (Attribute("csiter", &i) == 0) p["csiter"] = i;
            if (Attribute("cgiter", &i) == 0) p["nliter"] = i;
            if (Attribute("cgconv", &f) == 0) p["cgconv"] = f;
            if (Attribute("lsiter", &i) == 0) p["lsiter"] = i;
            p["ft"] = m_ft_type;
            if (const char *a = Configurable::Attribute("seed")) m_seed = (unsigned)std::atol(a);
            m_csx.reset(new CS_XSENSE<cxfl>(p));
            if (m_verbose) std::cout << *m_csx << std::endl;
        } catch (const codeare::error_code &e) {
            std::printf("**ERROR - CompressedSensing::Init: missing workspace matrix\n");
            return e;
        } catch (const std::exception &e) {
            std::printf("**ERROR - CompressedSensing::Init: %s\n", e.what());
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        }
        m_initialised = true;
        std::printf("... done.\n\n");
        return codeare::OK;
    }

    virtual codeare::error_code Prepare()
    {
        if (!m_csx) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            m_csx->KSpace(Get<float>("kspace"));
            m_csx->Weights(Get<float>("weights"));
        } catch (const codeare::error_code &e) {
            std::printf("**ERROR - CompressedSensing::Prepare: missing workspace matrix\n");
            return e;
        } catch (const std::exception &e) {
            std::printf("**ERROR - CompressedSensing::Prepare: %s\n", e.what());
            return codeare::CONTEXT_CONFIGURATION_FAILED;
        } catch (...) {
            std::printf("**ERROR - CompressedSensing::Prepare: bad k-space dimensions\n");
            return codeare::UNSUPPORTED_DIMENSION;
        }
        Free("weights");
        Free("kspace");
        return codeare::OK;
    }

    virtual codeare::error_code Process()
    {
        if (!m_initialised || !m_csx) return codeare::CONTEXT_CONFIGURATION_FAILED;
        try {
            Matrix<cxfl> data = m_test_case ? (*m_csx) * phantom<cxfl>(m_image_size[0]) : Get<cxfl>("data");
            if (m_noise > 0.f) {
                std::mt19937 gen(m_seed);
                std::normal_distribution<float> nd(0.f, 1.f);
                for (auto &v : data.Container()) v += m_noise * cxfl(nd(gen), nd(gen));
            }
            Matrix<cxfl> im_dc = (*m_csx)->*data;
            const cgs_cs_report &r = m_csx->LastReport();
            std::printf("  %d NLCG iterations, %d CG-SENSE solves, %.3f s on the GPU\n", r.iterations, r.solves,
                        r.seconds);
            if (m_verbose)
                for (int k = 0; k < r.iterations && k < 256; ++k)
                    std::printf("    %02d rmse %.6e  line search %d\n", k, r.rmse[k], r.ls_index[k]);
            Add("im_dc", im_dc);
        } catch (const codeare::error_code &e) {
            return e;
        } catch (const std::exception &e) {
            std::printf("**ERROR - CompressedSensing::Process: %s\n", e.what());
            return codeare::ERROR_GENERAL;
        }
        return codeare::OK;
    }

    virtual codeare::error_code Finalise()
    {
        m_csx.reset();
        return codeare::OK;
    }

private:
    // a list attribute ("8 8" or "8,8"), empty when absent (Configurable.hpp RHSList)
    std::vector<size_t> list(const char *key) const
    {
        std::vector<size_t> v;
        std::string s;
        if (Attribute(key, &s) != 0) return v;
        for (char &c : s)
            if (c == ',') c = ' ';
        std::istringstream is(s);
        size_t x;
        while (is >> x) v.push_back(x);
        return v;
    }

    std::unique_ptr<CS_XSENSE<cxfl>> m_csx;
    std::vector<size_t> m_image_size;
    size_t m_dim = 0;
    int m_verbose = 0, m_test_case = 0, m_ft_type = 3;
    float m_noise = 0.f;
    unsigned m_seed = 0;
};

}  // namespace RRStrategy

extern "C" DLLEXPORT RRStrategy::ReconStrategy *create() { return new RRStrategy::CompressedSensing; }
extern "C" DLLEXPORT void destroy(RRStrategy::ReconStrategy *p) { delete p; }
