// Reference-tree leaf order (placeholder until the GPU top-down build lands).
#include "sb_common.cuh"
#include "sb_internal.h"

namespace sbg {
sb_status build_reference_rank(sb_mesh *m, cudaStream_t)
{
    m->d.rankValid = false;
    return SB_OK;
}
} // namespace sbg
