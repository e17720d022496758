// Explicit instantiation of the half-sweep launchers for T = float, M = float
// (one translation unit per type pair so the build compiles them in parallel).
#include "sweep_impl.cuh"

namespace ginf_gpu {
template cudaError_t launch_sweep_tm<float, float>(const RecordFormat &, const SweepConfig &, const SweepParams &,
                                                cudaStream_t, int);
}  // namespace ginf_gpu
