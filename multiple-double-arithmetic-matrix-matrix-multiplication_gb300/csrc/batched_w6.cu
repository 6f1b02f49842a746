// Batched digit and renormalisation kernels with 6-word integers
// (see batched_stages.cuh).
#include "batched_stages.cuh"

template int mdgi::launch_batch_digits<6>(const mdgi::BatchProblem *, int, const int *, dim3,
                                           dim3, int, int, cudaStream_t);
template int mdgi::launch_batch_renorm<6>(int, const mdgi::BatchProblem *, int, const int *,
                                           int, int, int, cudaStream_t);
