// cgsense_run.cpp -- a minimal host that loads a ReconStrategy plugin the way
// codeare's ReconContext does (dlopen(name + ".so", RTLD_NOW), dlsym("create"),
// src/core/Loader.hpp.in:46-118, src/core/ReconContext.cpp:44-51) and drives
// Init / Prepare / Process / Finalise on workspace matrices read from a file.
//
//   cgsense_run <plugin.so> <config.xml> <inputs> <output> [output names...]
//
// <inputs> is a .cgsm container, or codeare .cod files named for the
// workspace: "sensitivities=s.cod,kspace=k.cod,...".  <output> is a .cgsm
// container, or a .cod file when exactly one output name is given.
//
// The .cgsm container holds named matrices: "CGSM" u32 count, then per entry
// u32 name length, name bytes, u32 type (0 float, 1 complex float), u32 ndims,
// u64 dims[ndims] (codeare order, first index fastest), raw data.  A .cod file
// (src/matrix/io/CODFile.hpp:103-190) holds one matrix: i32 type (0 float,
// 1 double, 2 complex float, 3 complex double), u64 ndims, u64 dims[ndims],
// f32 resolutions[ndims], u64 name length, name, data, then a 32-character
// delimiter.  Double data is converted to single precision.
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "codeare/ReconStrategy.hpp"

static bool read_cgsm(const char *path, Workspace &ws)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    char magic[4];
    uint32_t n = 0;
    f.read(magic, 4);
    f.read((char *)&n, 4);
    if (std::memcmp(magic, "CGSM", 4) != 0) return false;
    for (uint32_t e = 0; e < n; ++e) {
        uint32_t len = 0, type = 0, nd = 0;
        f.read((char *)&len, 4);
        std::string name(len, '\0');
        f.read(&name[0], len);
        f.read((char *)&type, 4);
        f.read((char *)&nd, 4);
        std::vector<size_t> dims(nd);
        for (uint32_t i = 0; i < nd; ++i) { uint64_t d; f.read((char *)&d, 8); dims[i] = (size_t)d; }
        if (type == 0) {
            Matrix<float> &m = ws.AddMatrix<float>(name);
            m = Matrix<float>(dims);
            f.read((char *)m.Ptr(), m.Size() * sizeof(float));
        } else {
            Matrix<cxfl> &m = ws.AddMatrix<cxfl>(name);
            m = Matrix<cxfl>(dims);
            f.read((char *)m.Ptr(), m.Size() * sizeof(cxfl));
        }
        if (!f) return false;
    }
    return true;
}

static const char kCodDelimiter[] = "543f562189f1e82beb9c177f89f67822";

static bool read_cod(const std::string &path, const std::string &name, Workspace &ws)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    int32_t dt = -1;
    uint64_t nd = 0, nlen = 0;
    f.read((char *)&dt, 4);
    f.read((char *)&nd, 8);
    if (!f || nd == 0 || nd > 16) return false;
    std::vector<size_t> dims(nd);
    size_t count = 1;
    for (uint64_t i = 0; i < nd; ++i) { uint64_t d; f.read((char *)&d, 8); dims[i] = (size_t)d; count *= (size_t)d; }
    std::vector<float> res(nd);
    f.read((char *)res.data(), 4 * nd);
    f.read((char *)&nlen, 8);
    if (!f || nlen > 4096) return false;
    std::string stored(nlen, '\0');
    f.read(&stored[0], (std::streamsize)nlen);
    if (dt == 0 || dt == 1) {
        Matrix<float> &m = ws.AddMatrix<float>(name);
        m = Matrix<float>(dims);
        if (dt == 0) {
            f.read((char *)m.Ptr(), count * sizeof(float));
        } else {
            std::vector<double> b(count);
            f.read((char *)b.data(), count * sizeof(double));
            for (size_t i = 0; i < count; ++i) m.Ptr()[i] = (float)b[i];
        }
    } else if (dt == 2 || dt == 3) {
        Matrix<cxfl> &m = ws.AddMatrix<cxfl>(name);
        m = Matrix<cxfl>(dims);
        if (dt == 2) {
            f.read((char *)m.Ptr(), count * sizeof(cxfl));
        } else {
            std::vector<double> b(2 * count);
            f.read((char *)b.data(), 2 * count * sizeof(double));
            for (size_t i = 0; i < count; ++i) m.Ptr()[i] = cxfl((float)b[2 * i], (float)b[2 * i + 1]);
        }
    } else {
        return false;
    }
    return (bool)f;
}

static bool write_cod(const char *path, Workspace &ws, const std::string &name)
{
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    auto header = [&](int32_t dt, const std::vector<size_t> &dims) {
        const uint64_t nd = dims.size(), nlen = name.size();
        f.write((const char *)&dt, 4);
        f.write((const char *)&nd, 8);
        for (size_t d : dims) { const uint64_t v = d; f.write((const char *)&v, 8); }
        for (size_t i = 0; i < dims.size(); ++i) { const float r = 1.f; f.write((const char *)&r, 4); }
        f.write((const char *)&nlen, 8);
        f.write(name.data(), (std::streamsize)nlen);
    };
    if (ws.Exists<cxfl>(name) == codeare::OK) {
        const Matrix<cxfl> &m = ws.Get<cxfl>(name);
        header(2, m.Dim());
        f.write((const char *)m.Ptr(), m.Size() * sizeof(cxfl));
    } else if (ws.Exists<float>(name) == codeare::OK) {
        const Matrix<float> &m = ws.Get<float>(name);
        header(0, m.Dim());
        f.write((const char *)m.Ptr(), m.Size() * sizeof(float));
    } else {
        return false;
    }
    f.write(kCodDelimiter, 32);
    return (bool)f;
}

static bool ends_with(const std::string &s, const char *suf)
{
    const size_t n = std::strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// "name=file.cod,name=file.cod,..."
static bool read_cod_list(const std::string &spec, Workspace &ws)
{
    std::stringstream ss(spec);
    std::string item;
    while (std::getline(ss, item, ',')) {
        const size_t eq = item.find('=');
        if (eq == std::string::npos || eq == 0) return false;
        if (!read_cod(item.substr(eq + 1), item.substr(0, eq), ws)) {
            std::fprintf(stderr, "cannot read %s\n", item.substr(eq + 1).c_str());
            return false;
        }
    }
    return true;
}

static bool write_cgsm(const char *path, Workspace &ws, const std::vector<std::string> &names)
{
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    f.write("CGSM", 4);
    uint32_t n = (uint32_t)names.size();
    f.write((const char *)&n, 4);
    for (const auto &name : names) {
        const Matrix<cxfl> &m = ws.Get<cxfl>(name);
        uint32_t len = (uint32_t)name.size(), type = 1, nd = (uint32_t)m.NDim();
        f.write((const char *)&len, 4);
        f.write(name.data(), len);
        f.write((const char *)&type, 4);
        f.write((const char *)&nd, 4);
        for (uint32_t i = 0; i < nd; ++i) { uint64_t d = m.Dim(i); f.write((const char *)&d, 8); }
        f.write((const char *)m.Ptr(), m.Size() * sizeof(cxfl));
    }
    return (bool)f;
}

int main(int argc, char **argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s plugin.so config.xml in.cgsm|name=f.cod,... out.cgsm|out.cod [outputs...]\n",
                     argv[0]);
        return 2;
    }
    std::ifstream cf(argv[2]);
    std::stringstream ss;
    ss << cf.rdbuf();
    const std::string xml = ss.str();
    Workspace &ws = Workspace::Instance();
    const std::string in(argv[3]);
    const bool cod_in = in.find('=') != std::string::npos;
    if (cod_in ? !read_cod_list(in, ws) : !read_cgsm(argv[3], ws)) {
        std::fprintf(stderr, "cannot read %s\n", argv[3]);
        return 3;
    }
    const bool cod_out = ends_with(argv[4], ".cod");
    if (cod_out && argc > 6) {
        std::fprintf(stderr, "a .cod output holds one matrix\n");
        return 2;
    }
    void *h = dlopen(argv[1], RTLD_NOW);
    if (!h) { std::fprintf(stderr, "dlopen: %s\n", dlerror()); return 4; }
    create_t *create = (create_t *)dlsym(h, "create");
    destroy_t *destroy = (destroy_t *)dlsym(h, "destroy");
    if (!create || !destroy) { std::fprintf(stderr, "plugin lacks create/destroy\n"); return 5; }
    RRStrategy::ReconStrategy *rs = create();
    {   // the module name is the plugin file's base name, as codeare's loader uses it
        std::string nm(argv[1]);
        const size_t sl = nm.find_last_of('/');
        if (sl != std::string::npos) nm = nm.substr(sl + 1);
        const size_t dot = nm.find('.');
        if (dot != std::string::npos) nm = nm.substr(0, dot);
        rs->Name(nm.c_str());
    }
    rs->WSpace(&ws);
    rs->SetConfig(xml.c_str());
    codeare::error_code e = rs->Init();
    if (e == codeare::OK) e = rs->Prepare();
    if (e == codeare::OK) e = rs->Process();
    if (e == codeare::OK) e = rs->Finalise();
    std::vector<std::string> outs;
    for (int i = 5; i < argc; ++i) outs.push_back(argv[i]);
    if (outs.empty()) outs.push_back("image");
    if (e == codeare::OK && !(cod_out ? write_cod(argv[4], ws, outs[0]) : write_cgsm(argv[4], ws, outs)))
        e = codeare::FILE_WRITE_FAILED;
    destroy(rs);
    ws.Clear();  // entries the plugin added carry deleters that live in the plugin
    dlclose(h);
    std::printf("cgsense_run: status %d\n", (int)e);
    return e == codeare::OK ? 0 : 10 + (int)e;
}
