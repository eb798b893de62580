// Thread-local error text; rrg_last_error / rrh_last_error read it.
#include "error.h"

#include "../../../include/rils_rols_gb300.h"
#include "../../../include/rils_rols_host.h"

namespace rrc {
namespace {
thread_local std::string g_error;
}
void set_error(const std::string& msg) { g_error = msg; }
const char* get_error() { return g_error.c_str(); }
}  // namespace rrc

extern "C" const char* rrg_last_error(void) { return rrc::get_error(); }
extern "C" const char* rrh_last_error(void) { return rrc::get_error(); }
extern "C" int32_t rrg_abi_version(void) { return RRG_ABI_VERSION; }
