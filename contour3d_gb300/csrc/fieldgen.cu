/*
 * fieldgen.cu -- device version of the seeded field generators of
 * fieldgen.h / fieldgen_cpu.c.  Mode tables are computed on the host with the
 * same functions; the per-node sums use the same operations in the same
 * order and the build disables contraction (-fmad=false), so the device
 * writes the same bytes as the host generator.
 */
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "fieldgen.h"

namespace {

__global__ void k_modes_f64(double* __restrict__ out, const double* __restrict__ tx, const double* __restrict__ ty,
                            const double* __restrict__ tz, const double* __restrict__ amp, int nmodes, long mx,
                            long my, long mz) {
  const long long n = (long long)mx * my * mz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long i = (long)(q % mx), j = (long)((q / mx) % my), k = (long)(q / ((long long)mx * my));
    double f = 0.0;
    for (int m = 0; m < nmodes; m++) {
      const double* ex = tx + 2 * ((size_t)m * mx + i);
      const double* ey = ty + 2 * ((size_t)m * my + j);
      const double* ez = tz + 2 * ((size_t)m * mz + k);
      f = f + c3d_mode_term(ex[0], ex[1], ey[0], ey[1], ez[0], ez[1], amp[m]);
    }
    out[q] = f;
  }
}

/* single-precision sums, stored as float, or widened to double (OUT = double) */
template <typename OUT>
__global__ void k_modes_f32(OUT* __restrict__ out, const double* __restrict__ tx, const double* __restrict__ ty,
                            const double* __restrict__ tz, const double* __restrict__ amp, int nmodes, long mx,
                            long my, long mz) {
  const long long n = (long long)mx * my * mz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long i = (long)(q % mx), j = (long)((q / mx) % my), k = (long)(q / ((long long)mx * my));
    float f = 0.0f;
    for (int m = 0; m < nmodes; m++) {
      const double* ex = tx + 2 * ((size_t)m * mx + i);
      const double* ey = ty + 2 * ((size_t)m * my + j);
      const double* ez = tz + 2 * ((size_t)m * mz + k);
      const float exr = (float)ex[0], exi = (float)ex[1], eyr = (float)ey[0], eyi = (float)ey[1],
                  ezr = (float)ez[0], ezi = (float)ez[1];
      const float tr = __fsub_rn(__fmul_rn(exr, eyr), __fmul_rn(exi, eyi));
      const float ti = __fadd_rn(__fmul_rn(exr, eyi), __fmul_rn(exi, eyr));
      f = __fadd_rn(f, __fmul_rn((float)amp[m], __fadd_rn(__fmul_rn(tr, ezi), __fmul_rn(ti, ezr))));
    }
    out[q] = (OUT)f;
  }
}

__global__ void k_blobs_f64(double* __restrict__ out, c3d_blobs_t b, long gx, long gy, long gz, long ox, long oy,
                            long oz, long mx, long my, long mz) {
  const long long n = (long long)mx * my * mz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long i = (long)(q % mx), j = (long)((q / mx) % my), k = (long)(q / ((long long)mx * my));
    const double x = (double)(i + ox) / (double)(gx - 1);
    const double y = (double)(j + oy) / (double)(gy - 1);
    const double z = (double)(k + oz) / (double)(gz - 1);
    out[q] = c3d_blobs_value(&b, x, y, z);
  }
}

int grid_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

/*
 * Fill a device buffer with the block [off, off + my) of a global Fourier
 * field (dtype 0 = f64, 1 = f32) at time `time`: every phase advances by
 * |k| * time turns (omega = |k|), as a solver's field evolves between
 * frames.  Returns the analytic std, or -1 on error.
 */
extern "C" double c3d_fieldgen_modes_device(void* out, int dtype, const long gl[3], const long off[3],
                                            const long my[3], int nmodes, int kmin, int kmax, double power,
                                            uint64_t seed, double time) {
  if (nmodes > C3D_MAX_MODES || nmodes < 1) return -1.0;
  c3d_modes_t* m = (c3d_modes_t*)malloc(sizeof(c3d_modes_t));
  if (!m) return -1.0;
  c3d_modes_init(m, nmodes, kmin, kmax, power, seed);
  if (time != 0.0) {
    for (int n = 0; n < nmodes; n++) {
      const double kk = (double)(m->kx[n] * m->kx[n] + m->ky[n] * m->ky[n] + m->kz[n] * m->kz[n]);
      double ph = m->phase[n] + sqrt(kk) * time;
      ph = ph - floor(ph);
      m->phase[n] = ph;
    }
  }
  const double std = m->std;
  std::vector<double> tab[3];
  for (int d = 0; d < 3; d++) tab[d].resize(2 * (size_t)nmodes * (size_t)my[d]);
  for (int n = 0; n < nmodes; n++) {
    const int kk[3] = {m->kx[n], m->ky[n], m->kz[n]};
    double pr, pi;
    c3d_sincos_turns(m->phase[n], &pi, &pr);
    for (int d = 0; d < 3; d++)
      for (long i = 0; i < my[d]; i++) {
        double re, im;
        c3d_mode_axis(kk[d], i + off[d], gl[d], &re, &im);
        if (d == 2) {
          const double r2 = re * pr - im * pi;
          const double i2 = re * pi + im * pr;
          re = r2;
          im = i2;
        }
        tab[d][2 * ((size_t)n * my[d] + i) + 0] = re;
        tab[d][2 * ((size_t)n * my[d] + i) + 1] = im;
      }
  }
  double* dt[4] = {nullptr, nullptr, nullptr, nullptr};
  int rc = 0;
  for (int d = 0; d < 3 && !rc; d++) {
    if (cudaMalloc(&dt[d], sizeof(double) * tab[d].size()) != cudaSuccess ||
        cudaMemcpy(dt[d], tab[d].data(), sizeof(double) * tab[d].size(), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = 1;
  }
  if (!rc && (cudaMalloc(&dt[3], sizeof(double) * nmodes) != cudaSuccess ||
              cudaMemcpy(dt[3], m->amp, sizeof(double) * nmodes, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = 1;
  if (!rc) {
    const long long n = (long long)my[0] * my[1] * my[2];
    if (dtype == 0)
      k_modes_f64<<<grid_blocks(n), 256>>>((double*)out, dt[0], dt[1], dt[2], dt[3], nmodes, my[0], my[1], my[2]);
    else
      k_modes_f32<float><<<grid_blocks(n), 256>>>((float*)out, dt[0], dt[1], dt[2], dt[3], nmodes, my[0], my[1],
                                                  my[2]);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = 1;
  }
  for (int d = 0; d < 4; d++)
    if (dt[d]) cudaFree(dt[d]);
  free(m);
  if (rc) {
    fprintf(stderr, "[CONTOUR3D ERROR] device field generation failed: %s\n", cudaGetErrorString(cudaGetLastError()));
    return -1.0;
  }
  return std;
}

/*
 * The same field launched on `stream` with stream-ordered scratch and no
 * device-wide synchronisation, so a solver can advance a resident field
 * while other work runs.  dtype 2: double storage of the single-precision
 * sums (dtype 1's values widened), a cheap stand-in for a solver's double
 * field on GPUs whose FP64 rate is low.  Returns the analytic std, or -1 on
 * error.
 */
extern "C" double c3d_fieldgen_modes_device_async(void* out, int dtype, const long gl[3], const long off[3],
                                                  const long my[3], int nmodes, int kmin, int kmax, double power,
                                                  uint64_t seed, double time, void* stream_v) {
  if (nmodes > C3D_MAX_MODES || nmodes < 1) return -1.0;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  c3d_modes_t* m = (c3d_modes_t*)malloc(sizeof(c3d_modes_t));
  if (!m) return -1.0;
  c3d_modes_init(m, nmodes, kmin, kmax, power, seed);
  for (int n = 0; n < nmodes && time != 0.0; n++) {
    const double kk = (double)(m->kx[n] * m->kx[n] + m->ky[n] * m->ky[n] + m->kz[n] * m->kz[n]);
    double ph = m->phase[n] + sqrt(kk) * time;
    m->phase[n] = ph - floor(ph);
  }
  const double std = m->std;
  const size_t nt = 2 * (size_t)nmodes * (size_t)(my[0] + my[1] + my[2]);
  std::vector<double> tab(nt + (size_t)nmodes);
  double* t3[3] = {tab.data(), tab.data() + 2 * (size_t)nmodes * my[0],
                   tab.data() + 2 * (size_t)nmodes * (my[0] + my[1])};
  for (int n = 0; n < nmodes; n++) {
    const int kk[3] = {m->kx[n], m->ky[n], m->kz[n]};
    double pr, pi;
    c3d_sincos_turns(m->phase[n], &pi, &pr);
    for (int d = 0; d < 3; d++)
      for (long i = 0; i < my[d]; i++) {
        double re, im;
        c3d_mode_axis(kk[d], i + off[d], gl[d], &re, &im);
        if (d == 2) {
          const double r2 = re * pr - im * pi;
          const double i2 = re * pi + im * pr;
          re = r2;
          im = i2;
        }
        t3[d][2 * ((size_t)n * my[d] + i) + 0] = re;
        t3[d][2 * ((size_t)n * my[d] + i) + 1] = im;
      }
  }
  for (int n = 0; n < nmodes; n++) tab[nt + n] = m->amp[n];
  free(m);
  double* d = nullptr;
  if (cudaMallocAsync(&d, sizeof(double) * tab.size(), stream) != cudaSuccess) return -1.0;
  int rc = cudaMemcpyAsync(d, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, stream) != cudaSuccess;
  if (!rc) {
    const double* dx = d;
    const double* dy = d + 2 * (size_t)nmodes * my[0];
    const double* dz = d + 2 * (size_t)nmodes * (my[0] + my[1]);
    const long long n = (long long)my[0] * my[1] * my[2];
    if (dtype == 0)
      k_modes_f64<<<grid_blocks(n), 256, 0, stream>>>((double*)out, dx, dy, dz, d + nt, nmodes, my[0], my[1], my[2]);
    else if (dtype == 2)
      k_modes_f32<double><<<grid_blocks(n), 256, 0, stream>>>((double*)out, dx, dy, dz, d + nt, nmodes, my[0], my[1],
                                                              my[2]);
    else
      k_modes_f32<float><<<grid_blocks(n), 256, 0, stream>>>((float*)out, dx, dy, dz, d + nt, nmodes, my[0], my[1],
                                                             my[2]);
    rc = cudaGetLastError() != cudaSuccess;
  }
  /* the pageable copy has been staged when cudaMemcpyAsync returned; the
     scratch is released in stream order after the kernel */
  cudaFreeAsync(d, stream);
  return rc ? -1.0 : std;
}

/* Gaussian-blob field (f64) into a device buffer; returns 0 or 1 */
extern "C" int c3d_fieldgen_blobs_device(double* out, const long gl[3], const long off[3], const long my[3],
                                         int nblobs, uint64_t seed) {
  if (nblobs < 1 || nblobs > C3D_MAX_BLOBS) return 1;
  c3d_blobs_t b;
  c3d_blobs_init(&b, nblobs, seed);
  const long long n = (long long)my[0] * my[1] * my[2];
  k_blobs_f64<<<grid_blocks(n), 256>>>(out, b, gl[0], gl[1], gl[2], off[0], off[1], off[2], my[0], my[1], my[2]);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
