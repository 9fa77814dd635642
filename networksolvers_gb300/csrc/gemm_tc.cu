// Split-precision GEMM on the tcgen05 tensor cores (placeholder until the kernel lands).
#include "nsg_internal.h"
namespace nsg {
bool gemm_split_tc(nsg_ctx*, const GemmArgs&) { return false; }
}  // namespace nsg
