// Batched exponent and digit kernels for batches whose widest problem needs
// 6-word integers, and the renormalisation of P = 4 (see
// batched_stages.cuh).
#include "batched_stages.cuh"

template int mdgi::launch_batch_scale<6>(const mdgi::BatchProblem *, int, int, int *,
                                          cudaStream_t);
template int mdgi::launch_batch_digits<6>(const mdgi::BatchProblem *, int, int, const int *,
                                           cudaStream_t);
template int mdgi::launch_batch_renorm<4>(const mdgi::BatchProblem *, int, int, int, int,
                                           const int *, cudaStream_t);
