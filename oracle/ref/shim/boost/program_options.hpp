// Build-only stand-in for the subset of boost::program_options that the reference's
// CModelAdapt::GetOptions declares (options_description, add_options chaining, value<T>
// with default_value / implicit_value). The oracle sets options through the OPTIONS struct and
// never parses a command line, so these types only need to compile.
#ifndef ORACLE_SHIM_BOOST_PO_HPP
#define ORACLE_SHIM_BOOST_PO_HPP
#include <string>
namespace boost { namespace program_options {
struct value_semantic { virtual ~value_semantic() {} };
template <class T> struct typed_value : value_semantic {
  explicit typed_value(T* p) : p_(p) {}
  typed_value* default_value(const T& v) { if (p_) *p_ = v; return this; }
  typed_value* default_value(const T& v, const std::string&) { if (p_) *p_ = v; return this; }
  typed_value* implicit_value(const T&) { return this; }
  typed_value* multitoken() { return this; }
  typed_value* composing() { return this; }
  T* p_;
};
template <class T> typed_value<T>* value(T* p = 0) { return new typed_value<T>(p); }
struct options_description;
struct options_description_easy_init {
  explicit options_description_easy_init(options_description* o) : o_(o) {}
  options_description_easy_init& operator()(const char*, const char*) { return *this; }
  options_description_easy_init& operator()(const char*, value_semantic* v, const char* = 0) { delete v; return *this; }
  options_description* o_;
};
struct options_description {
  options_description() {}
  explicit options_description(const std::string&) {}
  options_description_easy_init add_options() { return options_description_easy_init(this); }
  options_description& add(const options_description&) { return *this; }
};
}}  // namespace boost::program_options
#endif
