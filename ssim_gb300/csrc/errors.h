// errors.h -- exception types of the GB300 FEM library (host only).
#pragma once
#include <stdexcept>
#include <string>

namespace ssim_gb {

// ---------------------------------------------------------------- errors
struct cuda_error : std::runtime_error {
  explicit cuda_error(const std::string& s) : std::runtime_error(s) {}
};
struct invalid_argument : std::invalid_argument {
  explicit invalid_argument(const std::string& s) : std::invalid_argument(s) {}
};
struct state_error : std::runtime_error {
  explicit state_error(const std::string& s) : std::runtime_error(s) {}
};
struct numerical_error : std::runtime_error {
  explicit numerical_error(const std::string& s) : std::runtime_error(s) {}
};
struct device_timeout : std::runtime_error {
  explicit device_timeout(const std::string& s) : std::runtime_error(s) {}
};

// message returned by ssim_gb_last_error(NULL) on this thread (entry points without a handle)
void set_global_error(const std::string& msg);

}  // namespace ssim_gb
