// Fiber scheduler behind cuda_emu.h (test use only): runs the threads of each block as
// cooperative fibers in the calling OS thread, and resolves warp collectives and block barriers
// once every participant has arrived.  A launch whose fibers stop making progress (a collective
// that some lanes never reach) or that diverges (lanes of one warp at different intrinsics) ends
// with an error and a message instead of hanging.

#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cuda_emu.h"

EmuThread *emu_cur = nullptr;

struct EmuWarp {
  int size = 32;
  int arrived = 0;
  int op = 0;
  unsigned gen = 0;
  unsigned long long val[32], res[32];
  int arg[32];
};

struct EmuBlock {
  int size = 0;
  int arrived = 0;
  unsigned gen = 0;
  void *smem = nullptr;
};

namespace {

struct Fiber {
  ucontext_t ctx;
  EmuThread t;
  bool done = false;
};

constexpr size_t kStack = 256 * 1024;
ucontext_t g_sched;
Fiber *g_running = nullptr;
std::vector<char *> g_stacks;
void (*g_body)(void *) = nullptr;
void *g_ctx = nullptr;
long long g_progress = 0;
long long g_clock = 0;
bool g_failed = false;
std::string g_fail_msg;

void fiber_main() {
  g_body(g_ctx);
  g_running->done = true;
  g_progress++;
}  // returns to g_sched through uc_link

void yield_to_scheduler() { swapcontext(&g_running->ctx, &g_sched); }

// abandons the launch: the scheduler stops resuming this block's fibers
[[noreturn]] void fail_launch(const std::string &msg) {
  g_failed = true;
  g_fail_msg = msg;
  for (;;) yield_to_scheduler();
}

// a fresh context that runs fiber_main on `stack` and returns to the scheduler
__attribute__((noinline)) void start_fiber(Fiber &f, char *stack) {
  getcontext(&f.ctx);
  f.ctx.uc_stack.ss_sp = stack;
  f.ctx.uc_stack.ss_size = kStack;
  f.ctx.uc_link = &g_sched;
  makecontext(&f.ctx, fiber_main, 0);
}

}  // namespace

extern "C" const char *emu_last_failure(void) { return g_fail_msg.c_str(); }

unsigned long long emu_collective(int op, unsigned long long value, int arg) {
  EmuWarp *w = emu_cur->warp;
  const int lane = emu_cur->lane;
  if (w->arrived == 0) {
    w->op = op;
  } else if (w->op != op) {
    fail_launch("divergent warp: lanes at different warp intrinsics (op " + std::to_string(w->op) + " vs " +
                std::to_string(op) + ")");
  }
  w->val[lane] = value;
  w->arg[lane] = arg;
  w->arrived++;
  g_progress++;
  const unsigned gen = w->gen;
  if (w->arrived == w->size) {
    unsigned long long mask = 0;
    for (int l = 0; l < w->size; l++) mask |= (w->val[l] & 1ull) << l;
    for (int l = 0; l < w->size; l++) {
      int src = l;
      switch (op) {
        case EMU_SHFL: src = w->arg[l] & 31; break;
        case EMU_SHFL_XOR: src = (l ^ w->arg[l]) & 31; break;
        case EMU_SHFL_UP: src = l - w->arg[l] >= 0 ? l - w->arg[l] : l; break;
        default: break;
      }
      if (op == EMU_BALLOT) w->res[l] = mask;
      else if (op == EMU_ANY) w->res[l] = mask != 0;
      else if (op == EMU_SYNC) w->res[l] = 0;
      else w->res[l] = src < w->size ? w->val[src] : 0;
    }
    w->arrived = 0;
    w->gen++;
  } else {
    while (w->gen == gen) yield_to_scheduler();
  }
  return w->res[lane];
}

void emu_block_barrier() {
  EmuBlock *b = emu_cur->block;
  b->arrived++;
  g_progress++;
  const unsigned gen = b->gen;
  if (b->arrived == b->size) {
    b->arrived = 0;
    b->gen++;
  } else {
    while (b->gen == gen) yield_to_scheduler();
  }
}

void *emu_dynamic_smem() { return emu_cur->block->smem; }

long long emu_clock() { return ++g_clock; }

int emu_run(EmuDim3 grid, EmuDim3 block, size_t smem, void (*body)(void *), void *ctx) {
  const int nthreads = (int)(block.x * block.y * block.z);
  const long long nblocks = (long long)grid.x * grid.y * grid.z;
  if (nthreads <= 0 || nblocks <= 0) return 0;
  while ((int)g_stacks.size() < nthreads) g_stacks.push_back(static_cast<char *>(std::malloc(kStack)));
  g_body = body;
  g_ctx = ctx;
  g_failed = false;
  g_fail_msg.clear();
  std::vector<Fiber> fibers(nthreads);
  std::vector<EmuWarp> warps((nthreads + 31) / 32);
  std::vector<unsigned char> shared(smem ? smem : 1);
  for (long long bi = 0; bi < nblocks; bi++) {
    EmuBlock blk;
    blk.size = nthreads;
    std::fill(shared.begin(), shared.end(), 0);
    blk.smem = shared.data();
    for (size_t w = 0; w < warps.size(); w++) {
      warps[w] = EmuWarp();
      warps[w].size = std::min(32, nthreads - 32 * (int)w);
    }
    for (int i = 0; i < nthreads; i++) {
      Fiber &f = fibers[i];
      f.done = false;
      const unsigned tx = i % block.x, ty = (i / block.x) % block.y, tz = i / (block.x * block.y);
      const unsigned bx = (unsigned)(bi % grid.x), by = (unsigned)((bi / grid.x) % grid.y),
                     bz = (unsigned)(bi / ((long long)grid.x * grid.y));
      f.t = EmuThread{{tx, ty, tz}, {bx, by, bz}, block, grid, i % 32, &warps[i / 32], &blk};
      start_fiber(f, g_stacks[i]);
    }
    int done = 0;
    while (done < nthreads) {
      const long long before = g_progress;
      for (Fiber &f : fibers) {
        if (f.done) continue;
        emu_cur = &f.t;
        g_running = &f;
        swapcontext(&g_sched, &f.ctx);
        emu_cur = nullptr;
        if (g_failed) return 1;
        if (f.done) done++;
      }
      if (done < nthreads && g_progress == before) {
        g_fail_msg = "deadlock: " + std::to_string(nthreads - done) +
                     " threads wait at a warp intrinsic or barrier that the others never reach";
        return 1;
      }
    }
  }
  return 0;
}

int emu_unknown_kernel(const char *name) {
  g_fail_msg = std::string("kernel not emulated: ") + name;
  return 1;
}
