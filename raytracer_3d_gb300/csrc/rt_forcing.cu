// rt_forcing.cu -- set_forcing of the forced configurations on the GPU: an
// in-place update of the bottom z plane (Fortran k = 1) of E, applied before
// every step as the reference's main loop orders it (main.f90:69-70).
//
//   RT_FORCING_FLUX   E += dt*F/dzt(1)                 lee1.f90:199-212
//   RT_FORCING_RELAX  E -= dt*max(0,zdot)*(E-F)/dzt(1) critical_gm1.f90:125-139
//
// F is the interior of the reference's 5D forcing field (flux_lee / E_gm,
// axes x,y,k,l,m), x fastest.  zdot at Fortran z index 1 is the velocity of
// the right face of the bottom cell, i.e. vel[2] at z = 0.  The binary64
// form keeps the reference's operation order with explicit round-to-nearest
// operations (bit-identical to the oracle); the binary32 form evaluates the
// same expression in binary64 on the widened state and rounds once.
//
// The plane has nx*ny*nk*nl*nm cells (1/nz of the field); cell q of the
// plane is E cell (q mod nx*ny) + (q div nx*ny)*s[3], because (k,l,m) are
// the slowest axes of E.  The kernel is HBM bound: 2 reads and 1 write of
// the plane (plus zdot for RELAX).
#include <algorithm>

#include "../../include/rt_gb300.h"
#include "rt_kernels.h"

namespace rt {

namespace {

template <class T, int KIND>
__global__ void __launch_bounds__(256) forcing_kernel(T* __restrict__ E, const double* __restrict__ F,
                                                      const T* __restrict__ zdot, long long nxy,
                                                      long long nplane, long long s3, double dt, double dz) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nplane; q += stride) {
    const long long c = q % nxy + (q / nxy) * s3;
    const double e = (double)E[c];
    const double f = F[q];
    double r;
    if (KIND == RT_FORCING_FLUX) {
      r = dadd(e, ddiv(dmul(dt, f), dz));
    } else {
      const double w = fmax2(0.0, (double)zdot[c]);
      r = dsub(e, ddiv(dmul(dmul(dt, w), dsub(e, f)), dz));
    }
    E[c] = (T)r;
  }
}

template <class T, int KIND>
cudaError_t launch_kind(T* E, const double* F, const T* zdot, const Dims& d, double dt, double dz,
                        cudaStream_t st) {
  const long long nxy = (long long)d.n[0] * d.n[1];
  const long long nplane = nxy * d.nspec;
  if (nplane == 0) return cudaSuccess;
  const long long blocks = std::min<long long>((nplane + 255) / 256, 8LL * 152);
  forcing_kernel<T, KIND><<<(unsigned)blocks, 256, 0, st>>>(E, F, zdot, nxy, nplane, d.s[3], dt, dz);
  return cudaGetLastError();
}

}  // namespace

template <class T>
cudaError_t launch_forcing(T* E, const double* F, const T* zdot, const Dims& d, double dt, double dz,
                           int kind, cudaStream_t st) {
  if (kind == RT_FORCING_FLUX) return launch_kind<T, RT_FORCING_FLUX>(E, F, zdot, d, dt, dz, st);
  if (kind == RT_FORCING_RELAX) return launch_kind<T, RT_FORCING_RELAX>(E, F, zdot, d, dt, dz, st);
  return cudaErrorInvalidValue;
}

template cudaError_t launch_forcing<double>(double*, const double*, const double*, const Dims&, double, double,
                                            int, cudaStream_t);
template cudaError_t launch_forcing<float>(float*, const double*, const float*, const Dims&, double, double,
                                           int, cudaStream_t);

}  // namespace rt
