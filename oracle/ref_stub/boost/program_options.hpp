// Minimal stand-in for boost/program_options, written for this project.
//
// The reference's util/config.h parses command-line flags with
// boost::program_options. The reference build recipe in oracle/build_ref.sh
// only needs those declarations to compile: the harness in
// oracle/ref_driver.cpp fills the configuration struct directly and never
// parses a command line. Every call here is a no-op.
#pragma once
#include <ostream>
#include <string>
#include <vector>

namespace boost {
namespace program_options {

struct value_semantic {};

template <typename T>
value_semantic *value(T *) { return nullptr; }

struct options_description {
  explicit options_description(const std::string &) {}
  struct adder {
    adder &operator()(const char *, const char *) { return *this; }
    adder &operator()(const char *, value_semantic *, const char *) { return *this; }
  };
  adder add_options() { return adder(); }
};

inline std::ostream &operator<<(std::ostream &os, const options_description &) { return os; }

struct variables_map {
  std::size_t count(const std::string &) const { return 0; }
};

struct parsed_options {};

inline parsed_options parse_command_line(int, char **, const options_description &) {
  return parsed_options();
}
inline void store(const parsed_options &, variables_map &) {}
inline void notify(variables_map &) {}

}  // namespace program_options
}  // namespace boost
