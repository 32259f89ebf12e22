// Stand-in for Boost.PropertyTree (oracle build only): a flat list of
// key -> value strings with typed get/put, which is all the reference's
// Parameters class needs on the oracle path.
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
namespace boost { namespace property_tree {
struct ptree {
    using value_type = std::pair<std::string, ptree>;
    using iterator = std::vector<value_type>::iterator;
    using const_iterator = std::vector<value_type>::const_iterator;
    std::string data;
    std::vector<value_type> children;

    const_iterator find(const std::string& k) const {
        for (auto it = children.begin(); it != children.end(); ++it)
            if (it->first == k) return it;
        return children.end();
    }
    const_iterator not_found() const { return children.end(); }
    iterator begin() { return children.begin(); }
    iterator end() { return children.end(); }
    const_iterator begin() const { return children.begin(); }
    const_iterator end() const { return children.end(); }

    template <class T> T get(const std::string& k) const {
        auto it = find(k);
        if (it == children.end()) throw std::runtime_error("ptree: no key " + k);
        return parse<T>(it->second.data);
    }
    template <class T> T get(const std::string& k, const T& d) const {
        auto it = find(k);
        return it == children.end() ? d : parse<T>(it->second.data);
    }
    template <class T> void put(const std::string& k, const T& v) {
        for (auto& c : children)
            if (c.first == k) { c.second.data = format(v); return; }
        add(k, v);
    }
    template <class T> void add(const std::string& k, const T& v) {
        ptree child;
        child.data = format(v);
        children.emplace_back(k, child);
    }
    void add_child(const std::string& k, const ptree& c) { children.emplace_back(k, c); }
    const ptree& get_child(const std::string& k) const {
        auto it = find(k);
        if (it == children.end()) throw std::runtime_error("ptree: no child " + k);
        return it->second;
    }

private:
    template <class T> static T parse(const std::string& s) {
        std::istringstream is(s);
        T v{};
        is >> v;
        return v;
    }
    template <class T> static std::string format(const T& v) {
        std::ostringstream os;
        os.precision(17);
        os << v;
        return os.str();
    }
};
template <> inline std::string ptree::parse<std::string>(const std::string& s) { return s; }
} }
