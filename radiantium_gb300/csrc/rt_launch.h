/*
 * rt_launch.h - host-callable launchers of the kernels in rt_kernels.cu.
 */
#ifndef RT_LAUNCH_H
#define RT_LAUNCH_H
#include <cuda_runtime.h>
#include "rt_types.h"
#include "../../include/radiantium.h"

/* stats slots: 0 samples, 1 closest rays, 2 shadow rays, 3 node visits,
 * 4 primitive tests, 5 instance visits, 6 invalid samples */
cudaError_t rt_launch_render(const RtSceneView* S, const RtParams& P, float* samples, uint32_t* status,
                             unsigned long long* stats, bool counting, cudaStream_t stream);
cudaError_t rt_launch_accumulate(float* film, const float* samples, int64_t npix, int chunk_len, cudaStream_t stream);
cudaError_t rt_launch_finalize(float* out, const float* film, int64_t npix, float spp, cudaStream_t stream);
cudaError_t rt_launch_trace(const RtSceneView* S, const rt_ray* rays, int64_t n, rt_hit* hits, uint8_t* occ,
                            uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream,
                            bool wide = false);
/* device address of the fixed RT_NOALLOC_SCRATCH_BYTES scratch array on
 * `device`, which must be the current device; looked up once per device and
 * process (rt_noalloc.cu) */
cudaError_t rt_noalloc_scratch(int device, void** ptr);
/* adjoint (rt_adjoint.cu): gradients into grad_albedo / grad_alpha (accumulated) */
cudaError_t rt_launch_adjoint(const RtSceneView* S, const RtParams& P, int albedo_tex, const int* alpha_slot,
                              float* grad_albedo, float* grad_alpha, int n_alpha, const float* dLdI, uint32_t* status,
                              cudaStream_t stream);
/* light tracing (rt_particles.cu): particles [first, first + count) splatted into
 * `film` sums (one float4 per pixel); the record variant writes per-particle
 * splat slots instead; finish writes film * v + CameraTraceLight for every pixel */
cudaError_t rt_launch_particles(const RtSceneView* S, const RtParams& P, int64_t first, int64_t count, float4* film,
                                uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream);
cudaError_t rt_launch_particle_records(const RtSceneView* S, const RtParams& P, int64_t first, int64_t count,
                                       int32_t* rec_n, int32_t* rec_pix, float* rec_rgb, int rec_max,
                                       uint32_t* status, cudaStream_t stream);
cudaError_t rt_launch_particle_finish(const RtSceneView* S, int64_t npix, const float4* film, float v, float* out,
                                     uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream);
cudaError_t rt_launch_scale(float* v, int64_t n, float s, cudaStream_t stream);
cudaError_t rt_launch_env_sample(const RtSceneView* S, int which, const float2* u, int64_t n, int2* texel, float* pdf,
                                 cudaStream_t stream);
cudaError_t rt_launch_detmath(int fn, const float* a, const float* b, float* out, int64_t n, cudaStream_t stream);

#endif
