// Host-side launchers of the engine kernels (jdem_kernels.cu).
#pragma once
#include "jdem_device.cuh"

namespace jdem {

void launch_pack(int dim, const Bufs& b, const float* pos, const float* vel, const float* frc,
                 const float* rad, const float* mass, const int32_t* mat, const uint8_t* fixed,
                 const int32_t* sys_of, cudaStream_t st);
// Slot order -> caller order; a null destination skips that field.
void launch_unpack(int dim, const Bufs& b, float* pos, float* vel, float* frc, cudaStream_t st);
void launch_bbox_reset(const Bufs& b, cudaStream_t st);
void launch_identity_q(float4* q, long long n, cudaStream_t st);
void launch_scan_input(int dim, long long N, const float* pos, const float* rad, const int32_t* mat, int n_mat,
                       const int32_t* sys_of, unsigned int* out, cudaStream_t st);
void launch_default_inertia(int dim, long long N, const float* mass, const float* rad, float* inertia,
                            cudaStream_t st);
void launch_segcopy(const long long* seg, int nseg, int narr, const float* const* src, float* const* dst,
                    const int* width, cudaStream_t st);
void launch_scan(const Bufs& b, cudaStream_t st);
void launch_rebuild(int dim, const Bufs& b, bool any_free, cudaStream_t st);
void launch_pre(int dim, const Bufs& b, int mode, cudaStream_t st);
void launch_force(int dim, const Bufs& b, int mode, cudaStream_t st);
// Spheres without clumps or Cundall-Strack contacts (jdem_force2.cu, jdem_force3.cu).
template <int DIM>
void launch_force_dim(const Bufs& b, int mode, cudaStream_t st);
// Systems of at most this many slots use k_force_small (Bufs.small_lanes lanes a slot).
constexpr long long kSmallForceSlots = 32768;
// Many steps per launch for small systems (jdem_multi.cu): whether the handle
// qualifies (few enough slots to keep every block of the cooperative launch
// resident; not Cundall-Strack or clumps), the chunk's step count, and the
// cooperative k_multi that sets the while condition hw.  launch_multi returns
// nonzero when the launch fails.
bool multi_eligible(int dim, const Bufs& b, int device);
void launch_multi_init(const Bufs& b, unsigned int n, cudaStream_t st);
int launch_multi(int dim, const Bufs& b, cudaGraphConditionalHandle hw, cudaStream_t st);
// Cundall-Strack (jdem_cs.cu): force + torque kernel, then the integrating
// kernel unless mode is MODE_FORCE_ONLY; the rotational first-step phase.
void launch_cs(int dim, const Bufs& b, int mode, cudaStream_t st);
void launch_cs_rot_pre(int dim, const Bufs& b, cudaStream_t st);
// Rigid clumps (jdem_rigid.cu)
void launch_rb(int dim, const Bufs& b, int mode, cudaStream_t st);
void launch_rb_pre(int dim, const Bufs& b, int mode, cudaStream_t st);
void launch_rb_init(int dim, const Bufs& b, const float* pos, const float* vel, const float* frc, const float* rad,
                    const float* mass, const float4* q, const float* angv, const float* torque, const float* inertia,
                    const uint8_t* fixed, const int32_t* sys_of, float* world, cudaStream_t st);
void launch_rb_unpack(int dim, const Bufs& b, float* pos, float* vel, float* frc, float4* q, float* angv,
                      float* torque, bool per_sphere, cudaStream_t st);
void launch_rb_energy(int dim, const Bufs& b, double* out, cudaStream_t st);
// members' world positions pos_c + R(q) pos_p, caller order (pos: P x dim)
void launch_rb_world(int dim, const Bufs& b, float* pos, cudaStream_t st);
void launch_nlbuild(int dim, const Bufs& b, cudaStream_t st);
// brick list build (jdem_tiles.cu)
size_t tbuild_smem(int nst, int nv, int nrows);
int prepare_tbuild(size_t bytes);
void launch_tbuild(int dim, const Bufs& b, cudaStream_t st);
void launch_cond(const Bufs& b, cudaGraphConditionalHandle h, cudaStream_t st);
// After k_pre / k_force: fold the displacement into the bound (see k_fin).
void launch_fin(const Bufs& b, bool after_force, bool set_cond, cudaGraphConditionalHandle h, cudaStream_t st);
void launch_rot(int dim, const Bufs& b, const int32_t* sys_of, float4* q, float* angv, float* torque,
                const float* inertia, const uint8_t* fixed, long long nsteps, cudaStream_t st);
void launch_ke_rot(int dim, long long N, const float4* q, const float* angv, const float* inertia,
                   double* out, cudaStream_t st);
void launch_energy(int dim, const Bufs& b, double* out, cudaStream_t st);
void launch_contacts(int dim, const Bufs& b, int pass, int32_t* counts, const long long* offs,
                     int32_t* pairs, long long cap, cudaStream_t st);

}  // namespace jdem
