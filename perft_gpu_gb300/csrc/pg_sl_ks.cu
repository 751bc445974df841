// pg_sl_ks.cu -- kernels instantiated for the SlKS slider policy.
#include "pg_ops_impl.cuh"

namespace pg {
PG_DEFINE_OPS(SlKS, ks, PG_SLIDER_KOGGE_STONE)
}  // namespace pg

#include "pg_persist.cuh"

namespace pg {
cudaError_t persist_launch(const PersistArgs& a, cudaStream_t st, int num_sms, int* grid)
{
    return persist_launch_impl(a, st, num_sms, grid);
}
}  // namespace pg
