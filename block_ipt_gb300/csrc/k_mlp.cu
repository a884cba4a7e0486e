// k_mlp.cu - learned Davidson preconditioner.
#include "block_solver.h"
#include "common.cuh"

namespace iptgb {

LearnedCorrection *make_learned_correction(const float *params, cudaStream_t stream)
{
    (void)params; (void)stream;
    return nullptr;
}

}  // namespace iptgb
