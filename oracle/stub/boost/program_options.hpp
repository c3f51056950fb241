// Minimal stand-in for boost::program_options::variables_map, enough for the
// reference estimators' `args["name"].as<T>()` lookups when they are driven
// from the oracle harness. Test infrastructure only.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace boost {
namespace program_options {

class variable_value {
 public:
  variable_value() = default;
  template <class T>
  static variable_value of(const T& v) {
    variable_value r;
    r.p_ = std::make_shared<T>(v);
    return r;
  }
  template <class T>
  const T& as() const {
    return *static_cast<const T*>(p_.get());
  }

 private:
  std::shared_ptr<void> p_;
};

class variables_map : public std::map<std::string, variable_value> {};

}  // namespace program_options
}  // namespace boost
