// Exception-to-status translation for the C ABI.  Every extern "C" entry
// point runs its body through guarded(): C++ exceptions never cross the
// boundary; the message is kept per thread for gbba_last_error().
#pragma once

#include <new>
#include <stdexcept>
#include <string>

#include "../../include/gbba.h"
#include "device_buffer.h"

namespace gbba {

struct ApiError : std::runtime_error {
  int status;
  ApiError(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(int status, const std::string& msg);
int last_status();

template <typename F>
int guarded(F&& f) {
  try {
    f();
    set_last_error(GBBA_OK, "");
    return GBBA_OK;
  } catch (const ApiError& e) {
    set_last_error(e.status, e.what());
    return e.status;
  } catch (const CudaError& e) {
    set_last_error(GBBA_ERR_CUDA, e.what());
    return GBBA_ERR_CUDA;
  } catch (const std::out_of_range& e) {
    set_last_error(GBBA_ERR_OUT_OF_RANGE, e.what());
    return GBBA_ERR_OUT_OF_RANGE;
  } catch (const std::bad_alloc&) {
    set_last_error(GBBA_ERR_INTERNAL, "host allocation failed");
    return GBBA_ERR_INTERNAL;
  } catch (const std::exception& e) {
    set_last_error(GBBA_ERR_RUNTIME, e.what());
    return GBBA_ERR_RUNTIME;
  } catch (...) {
    set_last_error(GBBA_ERR_INTERNAL, "unknown exception");
    return GBBA_ERR_INTERNAL;
  }
}

}  // namespace gbba
