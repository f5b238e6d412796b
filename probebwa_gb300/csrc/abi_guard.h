// abi_guard.h -- no C++ exception crosses the C ABI. Host entry points run
// their bodies through these guards, which turn an exception (a failed host
// allocation above all: a vector the size of an input file) into a status
// and the text pbw_last_error returns.
#pragma once
#include <new>
#include <stdexcept>
#include <string>

#include "../../include/probebwa_gpu.h"

namespace pbw {

void set_handleless_error(const std::string& s);

template <class Report, class Body>
int guarded(const char* fn, Report&& report, Body&& body) {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    report(std::string(fn) + ": out of host memory");
    return PBW_ERR_NOMEM;
  } catch (const std::length_error& e) {
    report(std::string(fn) + ": input too large for host memory (" + e.what() + ")");
    return PBW_ERR_NOMEM;
  } catch (const std::exception& e) {
    report(std::string(fn) + ": " + e.what());
    return PBW_ERR_ARG;
  } catch (...) {
    report(std::string(fn) + ": unexpected failure");
    return PBW_ERR_ARG;
  }
}

// Entry points without a handle: the message goes to pbw_last_error(NULL).
template <class Body>
int guard_handleless(const char* fn, Body&& body) {
  return guarded(fn, [](const std::string& m) { set_handleless_error(m); }, body);
}

}  // namespace pbw
