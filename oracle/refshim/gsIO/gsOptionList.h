// Test-only stand-in for gismo's gsOptionList (typed key/value options with descriptions), so
// that the gsStructuralAnalysis solver headers compile unchanged for the CPU oracle.
#pragma once

#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

#include <gsCore/gsLinearAlgebra.h>

namespace gismo {

class gsOptionList {
public:
    enum updateType { ignoreIfUnknown = 0, addIfUnknown = 1 };

    void addInt(const std::string& k, const std::string&, index_t v) { ints[k] = v; }
    void addReal(const std::string& k, const std::string&, real_t v) { reals[k] = v; }
    void addSwitch(const std::string& k, const std::string&, bool v) { switches[k] = v; }
    void addString(const std::string& k, const std::string&, const std::string& v) { strings[k] = v; }

    index_t getInt(const std::string& k) const { return get(ints, k); }
    real_t getReal(const std::string& k) const { return get(reals, k); }
    bool getSwitch(const std::string& k) const { return get(switches, k); }
    std::string getString(const std::string& k) const { return get(strings, k); }

    index_t askInt(const std::string& k, index_t d = 0) const { return ask(ints, k, d); }
    real_t askReal(const std::string& k, real_t d = 0) const { return ask(reals, k, d); }
    bool askSwitch(const std::string& k, bool d = false) const { return ask(switches, k, d); }
    std::string askString(const std::string& k, const std::string& d = "") const { return ask(strings, k, d); }

    void setInt(const std::string& k, index_t v) { set(ints, k, v); }
    void setReal(const std::string& k, real_t v) { set(reals, k, v); }
    void setSwitch(const std::string& k, bool v) { set(switches, k, v); }
    void setString(const std::string& k, const std::string& v) { set(strings, k, v); }

    bool hasInt(const std::string& k) const { return ints.count(k) != 0; }
    bool hasReal(const std::string& k) const { return reals.count(k) != 0; }
    bool hasSwitch(const std::string& k) const { return switches.count(k) != 0; }
    bool hasString(const std::string& k) const { return strings.count(k) != 0; }

    void update(const gsOptionList& o, updateType mode = ignoreIfUnknown) {
        merge(ints, o.ints, mode);
        merge(reals, o.reals, mode);
        merge(switches, o.switches, mode);
        merge(strings, o.strings, mode);
    }

    friend std::ostream& operator<<(std::ostream& os, const gsOptionList& o) {
        for (auto& kv : o.ints) os << kv.first << " = " << kv.second << "\n";
        for (auto& kv : o.reals) os << kv.first << " = " << kv.second << "\n";
        for (auto& kv : o.switches) os << kv.first << " = " << kv.second << "\n";
        for (auto& kv : o.strings) os << kv.first << " = " << kv.second << "\n";
        return os;
    }

private:
    std::map<std::string, index_t> ints;
    std::map<std::string, real_t> reals;
    std::map<std::string, bool> switches;
    std::map<std::string, std::string> strings;

    template <class V>
    static V get(const std::map<std::string, V>& m, const std::string& k) {
        auto it = m.find(k);
        if (it == m.end()) throw std::runtime_error("option not found: " + k);
        return it->second;
    }
    template <class V>
    static V ask(const std::map<std::string, V>& m, const std::string& k, const V& d) {
        auto it = m.find(k);
        return it == m.end() ? d : it->second;
    }
    template <class V>
    static void set(std::map<std::string, V>& m, const std::string& k, const V& v) {
        auto it = m.find(k);
        if (it == m.end()) throw std::runtime_error("option not defined, cannot set: " + k);
        it->second = v;
    }
    template <class V>
    static void merge(std::map<std::string, V>& m, const std::map<std::string, V>& o, updateType mode) {
        for (auto& kv : o)
            if (m.count(kv.first) || mode == addIfUnknown) m[kv.first] = kv.second;
    }
};

}  // namespace gismo
