// mrsph_noalloc.cu — level-set sampling for callers that must not allocate.
//
// mrsph_sample_levelset stages its points and results in device buffers it
// allocates per call.  cudaMalloc/cudaFree synchronise the whole device and
// may be forbidden outright for a caller: code that runs while another
// library owns the device memory budget (a framework's caching allocator, a
// solver that reserved the device up front), code on a latency-critical path
// that cannot afford a device-wide synchronisation, or code inside a region
// where allocation is not allowed.  mrsph_sample_levelset_noalloc serves
// those callers: it stages through one fixed scratch array in device global
// memory that is part of the library image, so the call allocates nothing.
//
// The scratch array holds NOALLOC_MAX_POINTS points; every GPU that loads
// the library keeps it resident until the process exits.  All calls on a
// device share it, so calls that overlap on that GPU (from two host threads,
// or on two handles) race and must be serialised by the caller.  Each call
// overwrites every scratch word it reads back, so nothing needs clearing and
// the array simply keeps the last call's contents.
#include <cuda_runtime.h>

#include <mutex>

#include "handle.h"

namespace {

constexpr long long NOALLOC_MAX_POINTS = 65536;
constexpr int SLOT = 10;  // doubles per point: 3 in, 6 out, 1 for the integer tag

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_POINTS * SLOT];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
double* g_scratch_ptr[MAX_DEVICES] = {};

__global__ void k_tag_to_int(long long n, const double* __restrict__ out6, int* __restrict__ tag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) tag[i] = (int)out6[6 * i + 5];
}

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the array's host-side name is not a
// device address).
cudaError_t scratch_on(int dev, double** out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

int nfail(mrsph_handle* h, int code, const char* msg) {
  if (h) h->err = msg;
  return code;
}

}  // namespace

extern "C" int mrsph_sample_levelset_noalloc(mrsph_handle* h, long long n, const double* xyz, double* phi,
                                             double* norm, double* curv, int* tag) {
  if (!h) return MRSPH_ERR_ARG;
  if (!h->eng) return nfail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first");
  if (n <= 0 || !xyz) return nfail(h, MRSPH_ERR_ARG, "no points");
  if (n > NOALLOC_MAX_POINTS)
    return nfail(h, MRSPH_ERR_RANGE, "mrsph_sample_levelset_noalloc takes at most 65536 points per call");
  const int dev = h->prm.device;
  if (dev < 0 || dev >= MAX_DEVICES) return nfail(h, MRSPH_ERR_ARG, "device ordinal out of range");
  cudaError_t e = cudaSetDevice(dev);
  double* base = nullptr;
  if (e == cudaSuccess) e = scratch_on(dev, &base);
  if (e != cudaSuccess) {
    h->err = std::string("no-allocation scratch set-up: ") + cudaGetErrorString(e);
    return MRSPH_ERR_CUDA;
  }
  double* d_in = base;               // n x 3
  double* d_out = base + 3 * n;      // n x 6
  int* d_tag = (int*)(base + 9 * n); // n ints (fit in n doubles)
  cudaStream_t s = h->eng->stream();
  e = cudaMemcpyAsync(d_in, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int rc = h->eng->sample_device(n, d_in, d_out);
    if (rc) { h->err = h->eng->err; return rc; }
  }
  if (e == cudaSuccess && tag) {
    k_tag_to_int<<<(int)((n + 255) / 256), 256, 0, s>>>(n, d_out, d_tag);
    e = cudaGetLastError();
  }
  // scatter the interleaved results straight into the caller's arrays
  if (e == cudaSuccess && phi)
    e = cudaMemcpy2DAsync(phi, sizeof(double), d_out, 6 * sizeof(double), sizeof(double), n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && norm)
    e = cudaMemcpy2DAsync(norm, 3 * sizeof(double), d_out + 1, 6 * sizeof(double), 3 * sizeof(double), n,
                          cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && curv)
    e = cudaMemcpy2DAsync(curv, sizeof(double), d_out + 4, 6 * sizeof(double), sizeof(double), n,
                          cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && tag) e = cudaMemcpyAsync(tag, d_tag, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    h->err = std::string("mrsph_sample_levelset_noalloc: ") + cudaGetErrorString(e);
    return MRSPH_ERR_CUDA;
  }
  return 0;
}
