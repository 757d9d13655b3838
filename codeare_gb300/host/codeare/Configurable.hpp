// Configurable.hpp -- XML attribute access for plugins (reference:
// src/core/Configurable.hpp:52-475, backed by TinyXML).  This reader parses
// the attributes of the first element of the configuration fragment handed to
// SetConfig(), e.g. <CGSENSE nk="24576" lambda="0.05" cgmaxit="10"/>, and
// offers the same Attribute(name, T*) overloads, returning 0 when the key was
// found.  One deliberate difference: the reference writes an uninitialised
// double through Attribute(float*) when the key is absent
// (Configurable.hpp:311-318); here a missing key leaves the value unchanged.
#pragma once

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

class Configurable {
public:
    virtual ~Configurable() = default;

    // accepts an XML fragment; attributes of its first element are kept
    int SetConfig(const char *xml)
    {
        _attr.clear();
        if (!xml) return 1;
        const std::string s(xml);
        size_t p = s.find('<');
        while (p != std::string::npos && p + 1 < s.size() && (s[p + 1] == '?' || s[p + 1] == '!'))
            p = s.find('<', p + 1);
        if (p == std::string::npos) return 1;
        size_t q = p + 1;
        while (q < s.size() && !std::isspace((unsigned char)s[q]) && s[q] != '>' && s[q] != '/') ++q;
        _element = s.substr(p + 1, q - p - 1);
        while (q < s.size()) {
            while (q < s.size() && std::isspace((unsigned char)s[q])) ++q;
            if (q >= s.size() || s[q] == '>' || s[q] == '/') break;
            size_t eq = s.find('=', q);
            if (eq == std::string::npos) break;
            std::string key = s.substr(q, eq - q);
            while (!key.empty() && std::isspace((unsigned char)key.back())) key.pop_back();
            size_t v0 = eq + 1;
            while (v0 < s.size() && std::isspace((unsigned char)s[v0])) ++v0;
            if (v0 >= s.size() || (s[v0] != '"' && s[v0] != '\'')) break;
            const char quote = s[v0];
            size_t v1 = s.find(quote, v0 + 1);
            if (v1 == std::string::npos) break;
            _attr[key] = s.substr(v0 + 1, v1 - v0 - 1);
            q = v1 + 1;
        }
        return 0;
    }

    const std::string &Element() const { return _element; }

    void SetAttribute(const char *name, const std::string &value) { _attr[name] = value; }

    const char *Attribute(const char *name) const
    {
        auto it = _attr.find(name);
        return it == _attr.end() ? nullptr : it->second.c_str();
    }

    int Attribute(const char *name, std::string *v) const { return fetch(name, [&](const std::string &s) { *v = s; }); }
    int Attribute(const char *name, int *v) const { return fetch(name, [&](const std::string &s) { *v = std::atoi(s.c_str()); }); }
    int Attribute(const char *name, size_t *v) const { return fetch(name, [&](const std::string &s) { *v = (size_t)std::atol(s.c_str()); }); }
    int Attribute(const char *name, bool *v) const { return fetch(name, [&](const std::string &s) { *v = std::atoi(s.c_str()) != 0; }); }
    int Attribute(const char *name, double *v) const { return fetch(name, [&](const std::string &s) { *v = std::atof(s.c_str()); }); }
    int Attribute(const char *name, float *v) const { return fetch(name, [&](const std::string &s) { *v = (float)std::atof(s.c_str()); }); }

private:
    template <class F> int fetch(const char *name, F set) const
    {
        auto it = _attr.find(name);
        if (it == _attr.end()) {
            std::printf("**WARNING! Attribute '%s' does not exist in parameter list.\n", name);
            return 1;
        }
        set(it->second);
        return 0;
    }
    std::string _element;
    std::map<std::string, std::string> _attr;
};
