// Host emulation of the CUDA device-code constructs the engine's kernels use, for running those
// kernels on a CPU in tests (nothing here is part of the engine library).
//
// Every thread of a block is a cooperative fiber in one OS thread.  Warp-synchronous intrinsics
// (shuffles, ballots, __syncwarp) are collectives: a lane deposits its operand and yields until all
// 32 lanes of its warp have arrived at the same intrinsic, then every lane gets its result.
// __syncthreads does the same over the block.  Blocks run one after another.  Because fibers
// switch only at these points, atomics are plain read-modify-writes.  The engine's kernels use
// full-warp masks throughout; a collective reached by a partial warp or by different intrinsics
// is a divergence the emulator reports instead of guessing.
//
// Floating point: plain IEEE double operations (compile with -ffp-contract=off), which round to
// nearest like the *_rn intrinsics they stand in for.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __restrict__ __restrict
#define __align__(n) __attribute__((aligned(n)))
#define __launch_bounds__(...)
#define __shared__ static
#define __constant__

// vector types with the sizes and alignments of CUDA's
struct alignas(8) int2 {
  int x, y;
};
struct alignas(8) uint2 {
  unsigned int x, y;
};
struct alignas(16) int4 {
  int x, y, z, w;
};
struct alignas(16) uint4 {
  unsigned int x, y, z, w;
};
struct alignas(4) uchar4 {
  unsigned char x, y, z, w;
};
struct alignas(16) ulonglong2 {
  unsigned long long x, y;
};
static_assert(sizeof(int2) == 8 && sizeof(uint2) == 8 && sizeof(int4) == 16 && sizeof(uint4) == 16, "layout");
static_assert(sizeof(uchar4) == 4 && alignof(uchar4) == 4, "layout");
inline int2 make_int2(int x, int y) { return int2{x, y}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return uint2{x, y}; }
inline int4 make_int4(int x, int y, int z, int w) { return int4{x, y, z, w}; }
inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w) { return uint4{x, y, z, w}; }
inline ulonglong2 make_ulonglong2(unsigned long long x, unsigned long long y) { return ulonglong2{x, y}; }

struct EmuDim3 {
  unsigned x, y, z;
};

struct EmuWarp;
struct EmuBlock;

// the fiber that is running: its thread, block and grid coordinates
struct EmuThread {
  EmuDim3 tid, bid, bdim, gdim;
  int lane;
  EmuWarp *warp;
  EmuBlock *block;
};
extern EmuThread *emu_cur;

#define threadIdx (emu_cur->tid)
#define blockIdx (emu_cur->bid)
#define blockDim (emu_cur->bdim)
#define gridDim (emu_cur->gdim)

// ---- runtime (emu_runtime.cpp) ----
enum EmuOp { EMU_SYNC = 1, EMU_SHFL, EMU_SHFL_XOR, EMU_SHFL_UP, EMU_BALLOT, EMU_ANY };
unsigned long long emu_collective(int op, unsigned long long value, int arg);
void emu_block_barrier();
void *emu_dynamic_smem();
long long emu_clock();
// runs `body` as a grid of grid x block threads with `smem` bytes of dynamic shared memory per block;
// 0 when every thread returned, 1 when the launch failed (emu_last_failure() says why)
int emu_run(EmuDim3 grid, EmuDim3 block, size_t smem, void (*body)(void *), void *ctx);
extern "C" const char *emu_last_failure(void);
int emu_unknown_kernel(const char *name);  // records the failure and returns 1

// ---- intrinsics ----
template <class T>
inline unsigned long long emu_bits(T v) {
  static_assert(sizeof(T) <= 8, "64-bit operands at most");
  unsigned long long u = 0;
  std::memcpy(&u, &v, sizeof(T));
  return u;
}
template <class T>
inline T emu_from_bits(unsigned long long u) {
  T v;
  std::memcpy(&v, &u, sizeof(T));
  return v;
}

template <class T>
inline T __shfl_sync(unsigned, T v, int src) {
  return emu_from_bits<T>(emu_collective(EMU_SHFL, emu_bits(v), src));
}
template <class T>
inline T __shfl_xor_sync(unsigned, T v, int mask) {
  return emu_from_bits<T>(emu_collective(EMU_SHFL_XOR, emu_bits(v), mask));
}
template <class T>
inline T __shfl_up_sync(unsigned, T v, unsigned delta) {
  return emu_from_bits<T>(emu_collective(EMU_SHFL_UP, emu_bits(v), (int)delta));
}
inline unsigned __ballot_sync(unsigned, int pred) {
  return (unsigned)emu_collective(EMU_BALLOT, pred ? 1u : 0u, 0);
}
inline int __any_sync(unsigned, int pred) { return (int)emu_collective(EMU_ANY, pred ? 1u : 0u, 0); }
inline void __syncwarp(unsigned = 0xFFFFFFFFu) { emu_collective(EMU_SYNC, 0, 0); }
inline void __syncthreads() { emu_block_barrier(); }
inline unsigned emu_lanemask_lt() { return (1u << emu_cur->lane) - 1u; }

// device min/max (CUDA overloads them for integer arguments)
template <class A, class B>
inline std::common_type_t<A, B> max(A a, B b) {
  return a > b ? a : b;
}
template <class A, class B>
inline std::common_type_t<A, B> min(A a, B b) {
  return a < b ? a : b;
}

inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }
inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
inline double __dadd_rn(double a, double b) { return a + b; }
inline double __dsub_rn(double a, double b) { return a - b; }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __ddiv_rn(double a, double b) { return a / b; }
inline double __ll2double_rn(long long x) { return (double)x; }
inline double __ull2double_rn(unsigned long long x) { return (double)x; }
inline double __longlong_as_double(long long x) { return emu_from_bits<double>((unsigned long long)x); }
template <class T>
inline T __ldg(const T *p) {
  return *p;
}
inline long long clock64() { return emu_clock(); }

template <class T>
inline T atomicAdd(T *p, T v) {
  T old = *p;
  *p = old + v;
  return old;
}
template <class T>
inline T atomicMax(T *p, T v) {
  T old = *p;
  if (v > old) *p = v;
  return old;
}
template <class T>
inline T atomicExch(T *p, T v) {
  T old = *p;
  *p = v;
  return old;
}
template <class T>
inline T atomicOr(T *p, T v) {
  T old = *p;
  *p = old | v;
  return old;
}
template <class T>
inline T atomicCAS(T *p, T compare, T v) {
  T old = *p;
  if (old == compare) *p = v;
  return old;
}
