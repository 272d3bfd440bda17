// Minimal stand-in for the CAF header that the reference's src/cpu.cpp
// includes.  src/cpu.cpp uses CAF only for its command line (actor_system_config,
// opt_group, caf_main, CAF_MAIN); the WAH functions themselves are plain C++.
// With these empty declarations the reference file compiles unmodified, so the
// oracle can be checked against the reference's own code.  Test infrastructure
// only; nothing here is part of the product.
#pragma once
#include <string>

namespace caf {
struct config_option_set {};
struct actor_system_config {
  config_option_set custom_options_;
};
struct opt_group {
  opt_group(config_option_set&, const char*) {}
  template <class T>
  opt_group& add(T&, const char*, const char*) { return *this; }
};
struct actor_system {};
}  // namespace caf

// The reference ends with CAF_MAIN(); the shim provides its own entry points.
#define CAF_MAIN()
