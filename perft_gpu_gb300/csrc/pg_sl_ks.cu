// pg_sl_ks.cu -- kernels instantiated for the SlKS slider policy.
#include "pg_ops_impl.cuh"

namespace pg {
PG_DEFINE_OPS(SlKS, ks, PG_SLIDER_KOGGE_STONE)
}  // namespace pg
