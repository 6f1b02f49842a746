// Batched exponent and digit kernels for batches whose widest problem needs
// 4-word integers, and the renormalisation of P = 2 (see
// batched_stages.cuh).
#include "batched_stages.cuh"

template int mdgi::launch_batch_scale<4>(const mdgi::BatchProblem *, int, int, int *,
                                          cudaStream_t);
template int mdgi::launch_batch_digits<4>(const mdgi::BatchProblem *, int, int, const int *,
                                           cudaStream_t);
template int mdgi::launch_batch_renorm<2>(const mdgi::BatchProblem *, int, int, int, int,
                                           const int *, cudaStream_t);
