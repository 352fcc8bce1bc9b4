// rfgpu_fp64.cu - FP64 path.  Built with --fmad=false: every multiply and add
// rounds separately, as in the unfused Fortran expressions it restates, and
// the per-cell summation orders equal the reference's, so the residual and
// the stage update are bit-identical to the CPU restatement.
#include "rfgpu_kernels.cuh"
#include "rfmesh_stencil.h"

namespace rfgpu {

RFGPU_INSTANTIATE(double)

// WLSQ weights of RFLU_ComputeGradCellsFast_3D
// (modflu/RFLU_ModDifferentiationCells.F90:1022-1080), one thread per cell.
__global__ void k_weights64(const long long *__restrict__ stOff, const int *__restrict__ stCnt,
                            const int *__restrict__ stIdx, int N, long long T,
                            const double *__restrict__ cofg, const double *__restrict__ moms,
                            double *__restrict__ w) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  double r11 = moms[c], r12 = moms[N + c], r22 = moms[2 * N + c];
  double r13 = moms[3 * N + c], r23 = moms[4 * N + c], r33 = moms[5 * N + c];
  double c11 = 1.0 / r11, c22 = 1.0 / r22, c33 = 1.0 / r33;
  double c12 = -c11 * r12;
  double c13 = -(c11 * r13 + c12 * c22 * r23);
  double c23 = -c22 * r23;
  double c1111 = c11 * c11, c2222 = c22 * c22, c3333 = c33 * c33;
  double x0 = cofg[c], y0 = cofg[N + c], z0 = cofg[2 * N + c];
  long long e = stOff[c >> 5] + (c & 31);
  for (int k = 0; k < stCnt[c]; ++k, e += kSlice) {
    int nb = stIdx[e];
    double dx = cofg[nb] - x0, dy = cofg[N + nb] - y0, dz = cofg[2 * N + nb] - z0;
    double term = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
    dx = term * dx;
    dy = term * dy;
    dz = term * dz;
    double term1 = c1111 * (dx);
    double term2 = c2222 * (dy + c12 * dx);
    double term3 = c3333 * (dz + c23 * dy + c13 * dx);
    w[e] = term * (term1 + c12 * term2 + c13 * term3);
    w[T + e] = term * (term2 + c23 * term3);
    w[2 * T + e] = term * (term3);
  }
}

void launch_weights64(const long long *stOff, const int *stCnt, const int *stIdx, int nCells,
                      const double *cofg, const double *moms, double *w64, cudaStream_t s,
                      long long stTotal) {
  if (nCells <= 0) return;
  k_weights64<<<(nCells + 127) / 128, 128, 0, s>>>(stOff, stCnt, stIdx, nCells, stTotal, cofg,
                                                   moms, w64);
}

__global__ void k_to_f32(const double *__restrict__ src, float *__restrict__ dst, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < n; i += (long long)gridDim.x * blockDim.x) dst[i] = (float)src[i];
}

// c2c stencils and WLSQ moments of every cell, one thread per cell, with the
// per-cell routine the host mesh builder runs (rfmesh_stencil.h); this unit
// is built without contraction, so the moments match the host's bit for bit.
__global__ void __launch_bounds__(128) k_mesh_stencils(rfm::CellView m, int N, int *cnt, int *memb,
                                                       double *moms, int *overflow) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  rfm::Scratch w;
  int c2cs[rfm::kStencilMax];
  double mo[10];
  const int degr = rfm::cell_stencil(m, c, c2cs, mo, w);
  if (degr < 0) {
    atomicAdd(overflow, 1);
    cnt[c] = 0;
    return;
  }
  cnt[c] = degr;
  for (int s = 0; s < degr; ++s) memb[(size_t)c * rfm::kStencilMax + s] = c2cs[s];
  for (int k = 0; k < 10; ++k) moms[10 * (size_t)c + k] = mo[k];
}

void launch_mesh_stencils(const double *cofg, const int *cv, const int *nv, const int *v2cOff,
                          const int *v2c, int nCells, int *cnt, int *memb, double *moms,
                          int *overflow, cudaStream_t s) {
  if (nCells <= 0) return;
  rfm::CellView m{cofg, cv, nv, v2cOff, v2c};
  k_mesh_stencils<<<(nCells + 127) / 128, 128, 0, s>>>(m, nCells, cnt, memb, moms, overflow);
}

void launch_to_f32(const double *src, float *dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  long long blocks = (n + 255) / 256;
  if (blocks > 65535 * 8) blocks = 65535 * 8;
  k_to_f32<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n);
}

}  // namespace rfgpu

namespace rfgpu {

// Layout conversion between the Fortran image a(ncomp,N), host numbering,
// and device SoA in device numbering.  The loop runs over the host image, so
// its side of the copy is coalesced.
__global__ void k_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, int N,
                             int ncomp, const int *__restrict__ cellNew) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n = (long long)N * ncomp;
  for (; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long c = i / ncomp, k = i - c * ncomp;
    const long long cd = cellNew ? cellNew[c] : c;
    soa[k * N + cd] = aos[i];
  }
}

template <typename T>
__global__ void k_soa_to_aos(const T *__restrict__ soa, double *__restrict__ aos, int N, int ncomp,
                             const int *__restrict__ cellNew) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n = (long long)N * ncomp;
  for (; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long c = i / ncomp, k = i - c * ncomp;
    const long long cd = cellNew ? cellNew[c] : c;
    aos[i] = (double)soa[k * N + cd];
  }
}

static unsigned nblk(long long n) {
  long long b = (n + 255) / 256;
  return (unsigned)(b > 65535LL * 16 ? 65535LL * 16 : (b < 1 ? 1 : b));
}

void launch_aos_to_soa(const double *aos, double *soa, int N, int ncomp, const int *cellNew,
                       cudaStream_t s) {
  k_aos_to_soa<<<nblk((long long)N * ncomp), 256, 0, s>>>(aos, soa, N, ncomp, cellNew);
}
void launch_soa_to_aos(const double *soa, double *aos, int N, int ncomp, const int *cellNew,
                       cudaStream_t s) {
  k_soa_to_aos<double><<<nblk((long long)N * ncomp), 256, 0, s>>>(soa, aos, N, ncomp, cellNew);
}

template <typename T>
__global__ void k_grad_export(const T *__restrict__ g16, double *__restrict__ out, int N,
                              const int *__restrict__ cellNew) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n = (long long)N * 15;
  for (; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long c = i / 15, k = i - c * 15;
    const long long cd = cellNew ? cellNew[c] : c;
    out[i] = (double)g16[16 * cd + k];
  }
}

void launch_grad_export(const double *g16, double *out, int N, const int *cellNew,
                        cudaStream_t s) {
  k_grad_export<double><<<nblk((long long)N * 15), 256, 0, s>>>(g16, out, N, cellNew);
}
void launch_grad_export_f32(const float *g16, double *out, int N, const int *cellNew,
                            cudaStream_t s) {
  k_grad_export<float><<<nblk((long long)N * 15), 256, 0, s>>>(g16, out, N, cellNew);
}

}  // namespace rfgpu
