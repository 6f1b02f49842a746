// Batched exponent and digit kernels for batches whose widest problem needs
// 10-word integers, and the renormalisation of P = 8 (see
// batched_stages.cuh).
#include "batched_stages.cuh"

template int mdgi::launch_batch_scale<10>(const mdgi::BatchProblem *, int, int, int *,
                                          cudaStream_t);
template int mdgi::launch_batch_digits<10>(const mdgi::BatchProblem *, int, int, const int *,
                                           cudaStream_t);
template int mdgi::launch_batch_renorm<8>(const mdgi::BatchProblem *, int, int, int, int,
                                           const int *, cudaStream_t);
