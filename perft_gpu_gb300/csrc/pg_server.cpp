// pg_server.cpp -- continuous-batching perft server (host scheduler).
#include "../../include/perft_gb300.h"

extern "C" {
int pg_server_start(const pg_server_config*) { return PG_ERR_NOT_INITIALIZED; }
int pg_server_submit(const pg_board*, int, uint64_t*) { return PG_ERR_NOT_INITIALIZED; }
int pg_server_poll(uint64_t, uint64_t*, int*, double*) { return PG_ERR_NOT_INITIALIZED; }
int pg_server_stop(void) { return PG_OK; }
}
