// Tensor-core (tcgen05) path: placeholder until the BF16 kernels land.
#include "common.cuh"
#include "engine.h"

namespace gpunmf {
gpunmf_status tc_supported(int, int, int, int) {
    set_error("BF16 tensor-core path not built");
    return GPUNMF_ERR_UNSUPPORTED;
}
void tc_add_sizes(int, int, int, int, size_t *) {}
size_t tc_footprint(int, int, int, int) { return 0; }
gpunmf_status tc_create(gpunmf_job *) { return GPUNMF_ERR_UNSUPPORTED; }
gpunmf_status tc_prepare(gpunmf_job *) { return GPUNMF_ERR_UNSUPPORTED; }
gpunmf_status tc_iterate(gpunmf_job *, bool) { return GPUNMF_ERR_UNSUPPORTED; }
void tc_destroy(gpunmf_job *) {}
}  // namespace gpunmf
