// The window engine's kernels instantiated with integrator types 2-5 (EXT):
// Magnus CFET8, RK45 and RKF45 with quaternions, RKF45.  A run uses them when
// one of its parameter sets has such a type; every other run keeps the
// type 0/1 instantiations of st_kernels.cu, whose code and register budget
// these types do not touch.  The trajectory-ahead variants come with gas
// collisions only (they handle gas-free sets too).  Compiled as its own
// translation unit, in parallel with st_kernels.cu.
#include "st_engine.cuh"

namespace st {

const void* variant_fn_ext(int v) {
  switch (v) {
    case 0: return reinterpret_cast<const void*>(&k_persistent<128, 1, true>);
    case 1: return reinterpret_cast<const void*>(&k_persistent<128, 2, true>);
    case 2: return reinterpret_cast<const void*>(&k_persistent<128, 3, true>);
    case 3: return reinterpret_cast<const void*>(&k_persistent<64, 4, true>);
    case 4: return reinterpret_cast<const void*>(&k_persistent<256, 1, true>);
    case 5:
    case 6:
    case 19: return reinterpret_cast<const void*>(&k_batched<128, 1, 6, false, true, 0, true>);
    case 7: return reinterpret_cast<const void*>(&k_batched<128, 2, 4, false, true, 0, true>);
    case 12: return reinterpret_cast<const void*>(&k_batched<64, 2, 8, false, true, 1, true>);
    case 13: return reinterpret_cast<const void*>(&k_batched<64, 5, 6, false, true, 1, true>);
    case 21:
    case 22:
    case 23:
    case 24: return reinterpret_cast<const void*>(&k_batched<64, 2, 12, false, true, 0, true>);
    default: return reinterpret_cast<const void*>(&k_batched<64, 2, 8, false, true, 0, true>);  // 8 to 11, 20
  }
}

const void* tape_fn_ext() {
  return reinterpret_cast<const void*>(&k_batched<kTapeBlock, 1, kTapeQcap, true, true, 0, true>);
}

template <int B>
static int plain_launch_ext(const RunArgs& a, int window, double next_t, void* stream) {
  k_plain<B, true><<<(unsigned)((a.s.n + B - 1) / B), B, 0, (cudaStream_t)stream>>>(a, window, next_t);
  return (int)cudaGetLastError();
}

int launch_plain_ext(const RunArgs& a, int window, double next_t, int block, void* stream) {
  if (a.s.n == 0) return 0;
  if (block <= 32) return plain_launch_ext<32>(a, window, next_t, stream);
  if (block <= 64) return plain_launch_ext<64>(a, window, next_t, stream);
  if (block <= 128) return plain_launch_ext<128>(a, window, next_t, stream);
  return plain_launch_ext<256>(a, window, next_t, stream);
}

}  // namespace st
