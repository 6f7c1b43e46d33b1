// Error plumbing for the C ABI: library code throws ath::Error (or any
// std::exception); every exported function runs inside Guard(), which turns
// the exception into a status code and records its text for
// ath_last_error().  The library never calls exit().
#pragma once

#include <exception>
#include <stdexcept>
#include <string>

#include "aither_gb300.h"

namespace ath {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void SetError(const std::string &msg);
const char *LastError();

template <typename F>
int Guard(F &&f) {
  try {
    f();
    SetError("");
    return ATH_OK;
  } catch (const Error &e) {
    SetError(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    SetError("host out of memory");
    return ATH_ERR_NOMEM;
  } catch (const std::exception &e) {
    SetError(e.what());
    return ATH_ERR_IO;
  } catch (...) {
    SetError("unknown error");
    return ATH_ERR_IO;
  }
}

}  // namespace ath
