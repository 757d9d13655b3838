// ReconStrategy.hpp -- plugin base class (reference:
// src/core/ReconStrategy.hpp:47-255).  A plugin shared object exports
//   extern "C" ReconStrategy* create();  extern "C" void destroy(ReconStrategy*);
// and the host calls Name, WSpace, SetConfig, Init, Prepare, Process (any
// number of times), Finalise, then destroy.
#pragma once

#include <string>

#include "Configurable.hpp"
#include "Workspace.hpp"
#include "common.h"

#ifndef DLLEXPORT
#define DLLEXPORT __attribute__((visibility("default")))
#endif

namespace RRStrategy {

class ReconStrategy : public Configurable {
public:
    ReconStrategy() : m_initialised(false), global(nullptr) {}
    virtual ~ReconStrategy() {}

    virtual codeare::error_code Process() = 0;
    virtual codeare::error_code Init() = 0;
    virtual codeare::error_code Prepare() { return codeare::OK; }
    virtual codeare::error_code Finalise() { return codeare::OK; }

    void Name(const char *name) { m_name = std::string(name); }
    const char *Name() { return m_name.c_str(); }

    Workspace &DB() const { return *global; }
    void WSpace(Workspace *ws) { global = ws; }

    template <class T> Matrix<T> &Get(const std::string &name) const { return global->Get<T>(name); }
    template <class T> codeare::error_code Exists(const std::string &name) const { return global->Exists<T>(name); }
    bool Free(const std::string &name) const { return global->Free(name); }
    template <class T> void Add(const std::string &name, Matrix<T> &M) { global->Add(name, M); }
    template <class T> Matrix<T> &AddMatrix(const std::string &name) const { return global->AddMatrix<T>(name); }

protected:
    std::string m_name;
    bool m_initialised;
    Workspace *global;
};

}  // namespace RRStrategy

typedef RRStrategy::ReconStrategy *create_t();
typedef void destroy_t(RRStrategy::ReconStrategy *);
