// Compile-only stand-in for <boost/program_options.hpp>: TEST INFRASTRUCTURE
// ONLY.  The reference's Hamiltonian headers include its option-description
// helpers, which this oracle never calls; these declarations let those
// helpers compile (they build an options list that is never parsed).
#ifndef ORACLE_REF_STUB_BOOST_PROGRAM_OPTIONS_HPP
#define ORACLE_REF_STUB_BOOST_PROGRAM_OPTIONS_HPP

#include <map>
#include <string>

namespace boost {
namespace program_options {

struct value_semantic {
    virtual ~value_semantic() {}
};

template <class T>
struct typed_value : value_semantic {
    T v{};
    typed_value* default_value(const T& x) { v = x; return this; }
    typed_value* default_value(const T& x, const std::string&) { v = x; return this; }
    typed_value* multitoken() { return this; }
};

template <class T>
typed_value<T>* value() { return new typed_value<T>(); }

template <class T>
typed_value<T>* value(T*) { return new typed_value<T>(); }

struct options_description_easy_init {
    options_description_easy_init& operator()(const char*, const char*) { return *this; }
    options_description_easy_init& operator()(const char*, const value_semantic* v, const char* = "")
    {
        delete v;
        return *this;
    }
};

struct options_description {
    explicit options_description(const std::string& = "") {}
    options_description_easy_init add_options() { return {}; }
    options_description& add(const options_description&) { return *this; }
};

struct variable_value {
    template <class T>
    const T& as() const { static T x{}; return x; }
    bool empty() const { return true; }
};

struct variables_map : std::map<std::string, variable_value> {
    size_t count(const std::string&) const { return 0; }
};

}  // namespace program_options
}  // namespace boost

#endif
