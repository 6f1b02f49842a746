// Renormalisation kernels for P = 4 (see renorm_launch.cuh).
#include "renorm_launch.cuh"

template int mdgi::launch_renorm_p<4>(int, int, int, int, int, int, int, const int *, long long,
                                      int, const int *, const int *, double *, int, cudaStream_t);
