/*
 * refgpu.cu -- TEST INFRASTRUCTURE.  Compiles the reference's own device file
 * cuda_addon/particles_kernel.cu (included from the reference tree at build
 * time, never copied) into oracle/_ref/fcref_kernels.cubin for sm_103a, so
 * the reference's kernels can run on the same GPU and the same inputs as the
 * product kernels.  calcHashD, reorderDataAndFindCellStartD, collideD and the
 * __constant__ block `params` are used as the reference defines them; the one
 * wrapper below applies the reference's integrate_functor to element i, which
 * is what thrust::for_each over zip(pos4, vel4) does
 * (particleSystem.cu:141-153).
 */
#include <thrust/tuple.h>
#include "particles_kernel.cu"

extern "C" __global__ void fcref_integrate(float4 *pos, float4 *vel,
                                           float deltaTime, unsigned n) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  integrate_functor f(deltaTime);
  f(thrust::tie(pos[i], vel[i]));
}
