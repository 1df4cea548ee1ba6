/*
 * Precision form (FP32 bulk): placeholder until the FP32 kernels land.
 */
#include <cuda_runtime.h>

#include "nsem_mixed.h"

nsem_status nsem_mixed_setup(const NsemDev&, const nsem_mesh_desc*, NsemMixedBuf* mb,
                             std::vector<void*>*, std::string& err) {
    mb->ready = false;
    err = "precision form not built";
    return NSEM_UNSUPPORTED;
}

int nsem_mixed_steps(const NsemDev*, NsemMixedBuf*, NsemBuf*, const NsemTables*, int, double,
                     void*) {
    return (int)cudaErrorNotSupported;
}

int nsem_mixed_tendency(const NsemDev*, NsemMixedBuf*, NsemBuf*, const NsemTables*, void*) {
    return (int)cudaErrorNotSupported;
}

static const char* const k_names[] = {nullptr};
const char* const* nsem_mixed_kernel_names() { return k_names; }
int nsem_mixed_launches_per_step() { return 0; }
int nsem_mixed_launch_class(int) { return 0; }
int nsem_mixed_launch(const NsemDev*, NsemMixedBuf*, NsemBuf*, const NsemTables*, int, int, double,
                      void*) {
    return (int)cudaErrorNotSupported;
}
