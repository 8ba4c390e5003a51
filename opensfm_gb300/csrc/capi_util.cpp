#include "capi_util.h"

namespace gbba {

namespace {
thread_local std::string g_last_error;
thread_local int g_last_status = GBBA_OK;
}  // namespace

void set_last_error(int status, const std::string& msg) {
  g_last_status = status;
  g_last_error = msg;
}

int last_status() { return g_last_status; }

}  // namespace gbba

extern "C" const char* gbba_last_error(void) { return gbba::g_last_error.c_str(); }
