// pg_host_guard.h — the exception boundary of the C entry points.  Host code
// behind the C ABI uses the C++ library (vectors, strings, threads, locks), so
// an allocation that fails, a thread that cannot be started or a vector asked
// to exceed its maximum size raises a C++ exception; none may unwind into a C
// or JVM caller.  Each exported pg_status function is a function-try-block
// ending in PG_HOST_CATCH(obj), which turns the exception into a status and
// stores its description in obj->err (obj may be null).
#pragma once
#include <new>
#include <stdexcept>
#include <string>
#include <system_error>

#include "pilon_gb300.h"

namespace pg {

// Called inside a catch handler: the status for the exception being handled.
inline pg_status host_exception_status(std::string* err) noexcept {
  pg_status st = PG_ERR_NOMEM;
  const char* what = "host memory exhausted";
  try {
    throw;
  } catch (const std::bad_alloc&) {
  } catch (const std::length_error&) {
    st = PG_ERR_LIMIT;
    what = "a host buffer would exceed its maximum size";
  } catch (const std::system_error&) {
    what = "a host thread or lock could not be had";
  } catch (...) {
    what = "unexpected host exception";
  }
  if (err) {
    try {
      *err = what;
    } catch (...) {
    }
  }
  return st;
}

template <class T>
inline pg_status host_exception_status(T* obj) noexcept {
  return host_exception_status(obj ? &obj->err : nullptr);
}

}  // namespace pg

#define PG_HOST_CATCH(obj) \
  catch (...) {            \
    return pg::host_exception_status(obj); \
  }
