// Barriers for block-level routines that may run on a whole CTA or on a 128-thread group
// of a larger CTA (several groups then work independently, each on its own named barrier).
#pragma once

namespace ptg {
namespace {

struct SyncCta {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct SyncGroup128 {
  int id;   // 1..15 (0 is __syncthreads' barrier)
  __device__ __forceinline__ void operator()() const { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
};

}  // namespace
}  // namespace ptg
