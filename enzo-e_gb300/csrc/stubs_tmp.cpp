// temporary: batch and serving entry points land in batch.cu / serve.cpp
#include "../../include/mhdvlct_gb300.h"
extern "C" {
int mhdvlct_batch_create(mhdvlct_handle*, const int*, const double*, int, int, int, mhdvlct_batch**) { return MHD_ERR_INVALID; }
int mhdvlct_batch_destroy(mhdvlct_batch*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_block_view(mhdvlct_batch*, int, MhdBlockView*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_set_neighbors(mhdvlct_batch*, const int*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_refresh(mhdvlct_batch*, void*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_step(mhdvlct_batch*, const double*, void*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_timestep(mhdvlct_batch*, double*, void*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_run(mhdvlct_batch*, int, int, double*, void*) { return MHD_ERR_INVALID; }
int mhdvlct_batch_set_tile(mhdvlct_batch*, int, int) { return MHD_ERR_INVALID; }
int mhdserve_create(const MhdVlctParams*, size_t, int, mhdserve**) { return MHD_ERR_INVALID; }
int mhdserve_destroy(mhdserve*) { return MHD_ERR_INVALID; }
int mhdserve_submit(mhdserve*, const MhdServeRequest*, int*) { return MHD_ERR_INVALID; }
int mhdserve_pump(mhdserve*, int) { return MHD_ERR_INVALID; }
int mhdserve_poll(mhdserve*, int, int*) { return MHD_ERR_INVALID; }
int mhdserve_result(mhdserve*, int, float* const*, double*) { return MHD_ERR_INVALID; }
const char* mhdserve_last_error_string(const mhdserve*) { return "not built"; }
}
