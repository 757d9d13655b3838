// Params.hpp -- key/value parameter map passed from plugins to operators
// (reference: src/core/Params.hpp:168-371, a boost::any map; here std::any).
// Same access pattern: p["key"] = value; p.exists("key"); p.Get<T>("key")
// throws when the key is missing (the reference's KEY_NOT_FOUND) or the type
// differs (std::bad_any_cast in place of boost::bad_any_cast).
#pragma once

#include <any>
#include <cstddef>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

enum PARAMETER_MAP_EXCEPTION { KEY_NOT_FOUND };

class Params {
public:
    std::any &operator[](const std::string &key) { return _m[key]; }
    const std::any &operator[](const std::string &key) const
    {
        auto it = _m.find(key);
        if (it == _m.end()) throw KEY_NOT_FOUND;
        return it->second;
    }
    bool exists(const std::string &key) const { return _m.find(key) != _m.end(); }
    template <class T> T Get(const std::string &key) const { return std::any_cast<T>((*this)[key]); }
    template <class T> void Set(const std::string &key, const T &v) { _m[key] = v; }
    size_t size() const { return _m.size(); }

private:
    std::map<std::string, std::any> _m;
};

// numeric casts that accept any of the integer / floating types the reference
// stores for the same key (its unsigned_cast / fp_cast helpers)
inline size_t unsigned_cast(const std::any &a)
{
    if (a.type() == typeid(size_t)) return std::any_cast<size_t>(a);
    if (a.type() == typeid(int)) return (size_t)std::any_cast<int>(a);
    if (a.type() == typeid(unsigned)) return std::any_cast<unsigned>(a);
    if (a.type() == typeid(long)) return (size_t)std::any_cast<long>(a);
    if (a.type() == typeid(unsigned short)) return std::any_cast<unsigned short>(a);
    if (a.type() == typeid(float)) return (size_t)std::any_cast<float>(a);
    if (a.type() == typeid(double)) return (size_t)std::any_cast<double>(a);
    throw std::bad_any_cast();
}

inline double fp_cast(const std::any &a)
{
    if (a.type() == typeid(float)) return std::any_cast<float>(a);
    if (a.type() == typeid(double)) return std::any_cast<double>(a);
    if (a.type() == typeid(int)) return std::any_cast<int>(a);
    if (a.type() == typeid(size_t)) return (double)std::any_cast<size_t>(a);
    throw std::bad_any_cast();
}

template <class T> inline T try_to_fetch(const Params &p, const std::string &key, const T &def)
{
    if (!p.exists(key)) return def;
    try {
        if constexpr (std::is_integral<T>::value && !std::is_same<T, bool>::value) return (T)unsigned_cast(p[key]);
        else if constexpr (std::is_floating_point<T>::value) return (T)fp_cast(p[key]);
        else return p.Get<T>(key);
    } catch (const std::bad_any_cast &) {
        return def;
    }
}
