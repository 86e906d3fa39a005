// mcs_stubs.cpp -- placeholder C ABI entry points (filled in by later parts).
#include <string>

#include "../../include/mcsgpu.h"
#include "mcs_engine.h"

extern "C" {
struct mcs_server { int unused; };
static int unsupported(const char *what)
{
    mcs::set_error(std::string(what) + " is not built in this engine version");
    return MCS_EUNSUPPORTED;
}
int mcs_server_create(int32_t, uint64_t, int32_t, mcs_server **) { return unsupported("server"); }
int mcs_server_submit(mcs_server *, const mcs_problem *, const mcs_options *, uint64_t *) { return unsupported("server"); }
int mcs_server_step(mcs_server *, int32_t *) { return unsupported("server"); }
int mcs_server_poll(mcs_server *, uint64_t, mcs_result *) { return unsupported("server"); }
int mcs_server_stats(mcs_server *, int32_t *, int32_t *, uint64_t *, int64_t *) { return unsupported("server"); }
void mcs_server_destroy(mcs_server *) {}
}
