// Batched exponent and digit kernels for batches whose widest problem needs
// 16-word integers, and the renormalisation of P = 16 (see
// batched_stages.cuh).
#include "batched_stages.cuh"

template int mdgi::launch_batch_scale<16>(const mdgi::BatchProblem *, int, int, int *,
                                          cudaStream_t);
template int mdgi::launch_batch_digits<16>(const mdgi::BatchProblem *, int, int, const int *,
                                           cudaStream_t);
template int mdgi::launch_batch_renorm<16>(const mdgi::BatchProblem *, int, int, int, int,
                                           const int *, cudaStream_t);
