// ORACLE -- test infrastructure only (the reference's own CUDA kernels).
//
// Compiles the reference translation unit with its CUDA back end enabled
// (PRIMORDIAL_ROS2S_ENABLE_CUDA, reproducer.cpp:7372-7404) and without main, to a
// cubin for sm_103a.  The cubin then holds the reference's unmodified
// prepare_grid_timestep_kernel and advance_collapse_gridwide_kernel
// (reproducer.cpp:7696-7785), which oracle/ref_cuda_launcher.cpp runs on a GPU.
// Built by oracle/build_ref.sh WITH_CUBIN=1 where the reference tree is present;
// the flags are the reference's own (README.md:69): -O3 --fmad=false
// --maxrregcount=255 --expt-relaxed-constexpr.
//
// With -DPRIMORDIAL_ROS2S_CUDA_STRUCTURED (WITH_STRUCTURED=1) the same unit holds
// the reference's structured (gridwide-structured-cta32) advance kernel instead
// (structured_cuda.cuh:393-782, including the headers that the reference's own
// slicer tools/slice_dag.py generates); its shared-memory size is exported for the
// launcher as wr_ref_structured_shared_bytes.
#define PRIMORDIAL_ROS2S_ENABLE_CUDA 1
#define PRIMORDIAL_ROS2S_NO_MAIN 1
#include REFERENCE_TU
#if defined(PRIMORDIAL_ROS2S_CUDA_STRUCTURED)
extern "C" __device__ const unsigned long long wr_ref_structured_shared_bytes = structured_cuda::kSharedBytes;
#endif
