// Workspace.hpp -- named-matrix store shared by the host and the plugins
// (reference: src/core/Workspace.hpp:59-282, a singleton of shared_ptr'd
// matrices).  Same calls: Instance(), Get<T>(name), Add(name, M),
// AddMatrix<T>(name), Free(name), Exists<T>(name).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <typeinfo>

#include "Matrix.hpp"
#include "common.h"

class Workspace {
public:
    static Workspace &Instance()
    {
        static Workspace ws;
        return ws;
    }

    template <class T> Matrix<T> &Get(const std::string &name)
    {
        auto it = _store.find(name);
        if (it == _store.end() || *it->second.type != typeid(Matrix<T>)) throw codeare::NO_MATRIX_IN_WORKSPACE_BY_NAME;
        return *static_cast<Matrix<T> *>(it->second.ptr.get());
    }

    template <class T> codeare::error_code Exists(const std::string &name) const
    {
        auto it = _store.find(name);
        if (it == _store.end()) return codeare::NO_MATRIX_IN_WORKSPACE_BY_NAME;
        return (*it->second.type == typeid(Matrix<T>)) ? codeare::OK : codeare::WRONG_MATRIX_TYPE;
    }

    template <class T> Matrix<T> &AddMatrix(const std::string &name)
    {
        Entry e;
        e.ptr = std::shared_ptr<void>(new Matrix<T>(), [](void *p) { delete static_cast<Matrix<T> *>(p); });
        e.type = &typeid(Matrix<T>);
        _store[name] = e;
        return *static_cast<Matrix<T> *>(e.ptr.get());
    }

    template <class T> void Add(const std::string &name, const Matrix<T> &m) { AddMatrix<T>(name) = m; }

    bool Free(const std::string &name) { return _store.erase(name) > 0; }
    void Clear() { _store.clear(); }

private:
    struct Entry {
        std::shared_ptr<void> ptr;
        const std::type_info *type = nullptr;
    };
    Workspace() = default;
    std::map<std::string, Entry> _store;
};
