// A CPU runtime for the kernels of fortrancfd_gb300/csrc/fluid.cu (test
// infrastructure). Each thread of a CTA is a fiber (ucontext); the
// scheduler runs the fibers until each waits at __syncthreads, at a warp
// barrier (__syncwarp and the two halves of a shuffle) or has returned, and
// releases a barrier once every thread it names has arrived, so the kernels
// run with their own synchronisation. CTAs run one after another; shared
// memory is filled with NaN (or, EMU_POISON=big / zero, with +-1e300 or 0)
// before each, so a read of shared memory that no thread of the CTA wrote
// shows up. The few CUDA runtime calls of fluid.cu's
// host code are stubs (no device exists): memory is host memory, streams
// are ignored, constant-memory uploads are copies.
#pragma once
#include <cuda_runtime_api.h>
#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <vector>

#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif

struct EmuIdx {
  unsigned x = 0, y = 0, z = 0;
};
struct EmuFiber {
  ucontext_t ctx;
  int tid = 0;
  int state = 0;  // 0 runnable, 1 at __syncthreads, 2 at a warp barrier, 3 returned
  unsigned wmask = 0;
  std::vector<char> stack;
};
static std::vector<EmuFiber> emu_f;
static ucontext_t emu_sched;
static int emu_cur = 0;
static EmuIdx emu_block, emu_bdim, emu_gdim;
static inline EmuIdx emu_tidx() {
  EmuIdx e;
  e.x = emu_f[emu_cur].tid;
  return e;
}
#define threadIdx (emu_tidx())
#define blockIdx emu_block
#define blockDim emu_bdim
#define gridDim emu_gdim

static double emu_dslot[1024];
static int emu_islot[1024];
static int emu_bar_or = 0;
static double emu_sm[1 << 17];

static void emu_wait(int st, unsigned mask = 0) {
  emu_f[emu_cur].state = st;
  emu_f[emu_cur].wmask = mask;
  swapcontext(&emu_f[emu_cur].ctx, &emu_sched);
}
inline void __syncthreads() { emu_wait(1); }
inline int __syncthreads_or(int v) {
  if (v) emu_bar_or = 1;
  emu_wait(1);
  const int r = emu_bar_or;
  emu_wait(1);
  emu_bar_or = 0;
  return r;
}
inline void __syncwarp(unsigned mask = 0xffffffffu) { emu_wait(2, mask); }
inline double __shfl_xor_sync(unsigned mask, double v, int o, int = 32) {
  const int t = emu_f[emu_cur].tid, lane = t & 31;
  emu_dslot[t] = v;
  emu_wait(2, mask);
  const double r = emu_dslot[t - lane + (lane ^ o)];
  emu_wait(2, mask);
  return r;
}
inline int __shfl_up_sync(unsigned mask, int v, int d, int = 32) {
  const int t = emu_f[emu_cur].tid, lane = t & 31;
  emu_islot[t] = v;
  emu_wait(2, mask);
  const int r = lane >= d ? emu_islot[t - d] : v;
  emu_wait(2, mask);
  return r;
}
inline int __double2loint(double x) {
  unsigned long long v;
  std::memcpy(&v, &x, 8);
  return (int)(unsigned)(v & 0xffffffffull);
}
inline int __double2hiint(double x) {
  unsigned long long v;
  std::memcpy(&v, &x, 8);
  return (int)(unsigned)(v >> 32);
}
inline double __hiloint2double(int hi, int lo) {
  const unsigned long long v = ((unsigned long long)(unsigned)hi << 32) | (unsigned)lo;
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline long long __double_as_longlong(double x) {
  long long v;
  std::memcpy(&v, &x, 8);
  return v;
}
inline double __longlong_as_double(long long v) {
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __dadd_rn(double a, double b) { return a + b; }
inline double __dsub_rn(double a, double b) { return a - b; }
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline unsigned atomicOr(unsigned* p, unsigned v) {
  const unsigned o = *p;
  *p |= v;
  return o;
}
inline int atomicOr(int* p, int v) {
  const int o = *p;
  *p |= v;
  return o;
}
inline unsigned long long atomicMax(unsigned long long* p, unsigned long long v) {
  const unsigned long long o = *p;
  if (v > o) *p = v;
  return o;
}
inline int atomicAdd(int* p, int v) {
  const int o = *p;
  *p += v;
  return o;
}
inline unsigned atomicAdd(unsigned* p, unsigned v) {
  const unsigned o = *p;
  *p += v;
  return o;
}
using std::fma;
using std::max;
using std::min;
using std::sqrt;

// The value unwritten shared memory holds: NaN by default; EMU_POISON=big
// (alternating +-1e300) or EMU_POISON=zero instead, since a NaN can vanish
// in fmin / fmax (minmod limiters) where a large stale value would not.
static double emu_poison() {
  static int mode = -1;
  static unsigned long long k = 0;
  if (mode < 0) {
    const char* e = std::getenv("EMU_POISON");
    mode = !e ? 0 : (std::strcmp(e, "big") == 0 ? 1 : std::strcmp(e, "zero") == 0 ? 2 : 0);
  }
  if (mode == 1) return (k++ & 1) ? 1e300 : -1e300;
  if (mode == 2) return 0.0;
  return std::numeric_limits<double>::quiet_NaN();
}

static std::function<void()> emu_body;
static void emu_entry() {
  emu_body();
  emu_f[emu_cur].state = 3;
  swapcontext(&emu_f[emu_cur].ctx, &emu_sched);
}

// one CTA of nt threads through fn
static void emu_run_cta(int nt, const std::function<void()>& fn) {
  for (double& x : emu_sm) x = emu_poison();
  if ((int)emu_f.size() != nt) emu_f.assign(nt, EmuFiber());
  emu_body = fn;
  for (int t = 0; t < nt; ++t) {
    EmuFiber& f = emu_f[t];
    f.tid = t;
    f.state = 0;
    f.stack.resize(1 << 17);
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack.data();
    f.ctx.uc_stack.ss_size = f.stack.size();
    f.ctx.uc_link = nullptr;
    makecontext(&f.ctx, emu_entry, 0);
  }
  for (;;) {
    bool ran = false;
    for (int t = 0; t < nt; ++t)
      if (emu_f[t].state == 0) {
        emu_cur = t;
        swapcontext(&emu_sched, &emu_f[t].ctx);
        ran = true;
      }
    if (ran) continue;
    bool released = false;
    for (int w = 0; w * 32 < nt; ++w)
      for (int l = 0; l < 32 && w * 32 + l < nt; ++l) {
        if (emu_f[w * 32 + l].state != 2) continue;
        const unsigned m = emu_f[w * 32 + l].wmask;
        bool all = true;
        for (int b = 0; b < 32 && all; ++b)
          if (m & (1u << b)) {
            const int q = w * 32 + b;
            all = q < nt && emu_f[q].state == 2 && emu_f[q].wmask == m;
          }
        if (all) {
          for (int b = 0; b < 32; ++b)
            if (m & (1u << b)) emu_f[w * 32 + b].state = 0;
          released = true;
        }
      }
    if (released) continue;
    bool live = false, at_barrier = true;
    for (int t = 0; t < nt; ++t) {
      if (emu_f[t].state == 3) continue;
      live = true;
      if (emu_f[t].state != 1) at_barrier = false;
    }
    if (!live) break;
    if (at_barrier) {
      for (int t = 0; t < nt; ++t)
        if (emu_f[t].state == 1) emu_f[t].state = 0;
      continue;
    }
    std::fprintf(stderr, "CTA emulation: threads wait at barriers that cannot all be met\n");
    std::abort();
  }
}

template <class K, class... A>
static void emu_launch(K k, dim3 grid, dim3 block, size_t, cudaStream_t, A... args) {
  emu_gdim.x = grid.x;
  emu_gdim.y = grid.y;
  emu_bdim.x = block.x;
  for (unsigned y = 0; y < grid.y; ++y)
    for (unsigned b = 0; b < grid.x; ++b) {
      emu_block.x = b;
      emu_block.y = y;
      emu_run_cta((int)block.x, [&] { k(args...); });
    }
}

extern "C" {
cudaError_t cudaFuncSetAttribute(const void*, enum cudaFuncAttribute, int) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int* n, const void*, int, size_t) {
  *n = 2;
  return cudaSuccess;
}
cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(int* n, const void*, int, size_t, unsigned) {
  *n = 2;
  return cudaSuccess;
}
cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
cudaError_t cudaDeviceGetAttribute(int* v, enum cudaDeviceAttr, int) {
  *v = 152;
  return cudaSuccess;
}
cudaError_t cudaMemcpyToSymbolAsync(const void* sym, const void* src, size_t n, size_t off, enum cudaMemcpyKind,
                                    cudaStream_t) {
  std::memcpy((char*)sym + off, src, n);
  return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t) {
  std::memset(p, v, n);
  return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "CTA emulation"; }
}
template <class T>
cudaError_t cudaMemcpyToSymbolAsync(const T& sym, const void* src, size_t n, size_t off = 0,
                                    enum cudaMemcpyKind = cudaMemcpyHostToDevice, cudaStream_t = 0) {
  std::memcpy((char*)&sym + off, src, n);
  return cudaSuccess;
}
template <class T>
cudaError_t cudaFuncSetAttribute(T*, enum cudaFuncAttribute, int) {
  return cudaSuccess;
}
