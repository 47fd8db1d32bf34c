/* ref_cuda_kernels.cu -- TEST INFRASTRUCTURE ONLY.
 *
 * One translation unit that compiles the reference's own CUDA kernels where
 * they lie: sixtracklib/cuda/kernels/track_particles.cu (until-turn, line
 * and element-by-element tracking, each with its debug variant) and
 * sixtracklib/cuda/kernels/managed_buffer_remap.cu (the device-side buffer
 * remap the reference runs before tracking).  oracle/build_ref_cuda.sh
 * builds it for sm_103a with the reference's release flags into
 * oracle/_ref/ref_track_sm103a.cubin; oracle/ref_cuda.py loads and launches
 * it as a second GPU baseline and a parity pin for the engine.
 */
#include "sixtracklib/cuda/kernels/track_particles.cu"
#include "sixtracklib/cuda/kernels/managed_buffer_remap.cu"
