// jfem_abi_guard.h — the exception barrier of the C ABI.
//
// The library's host code is C++ (std::vector scratch of the mesh, tile and
// coarse-space builders, std::thread workers, std::string messages), while its
// callers are C, ctypes or Julia's ccall, none of which can catch a C++
// exception: one that crossed an extern "C" function would end the caller's
// process.  So every entry point runs its body between ABI_TRY and ABI_CATCH,
// which turn a host allocation failure (std::bad_alloc) or a thread or mutex
// that cannot be created (std::system_error) into JFEM_ERR_OOM, and anything
// else into JFEM_ERR_INVALID, with the message stored where the entry point's
// last-error string lives.  Device state is left as the failing step left it;
// the builders that mutate state in several steps (mesh, surface loads, coarse
// space) leave it empty or marked for rebuild on any failure.
#pragma once

#include <exception>
#include <new>
#include <string>
#include <system_error>

#include "../../include/jfem.h"

namespace jfem {

// Classifies the exception being handled (call only inside a catch block).
inline int host_exception_status(std::string* msg) noexcept {
  int code = JFEM_ERR_INVALID;
  const char* what = "unexpected host exception";
  try {
    throw;
  } catch (const std::bad_alloc&) {
    code = JFEM_ERR_OOM;
    what = "host memory exhausted";
  } catch (const std::system_error&) {
    code = JFEM_ERR_OOM;
    what = "host threads or locks unavailable";
  } catch (const std::exception& e) {
    what = e.what();
  } catch (...) {
  }
  if (msg) {
    try {
      *msg = what;
    } catch (...) {
    }
  }
  return code;
}

}  // namespace jfem

#define ABI_TRY try {
#define ABI_CATCH(msg_ptr)                          \
  }                                                 \
  catch (...) {                                     \
    return jfem::host_exception_status(msg_ptr);    \
  }
