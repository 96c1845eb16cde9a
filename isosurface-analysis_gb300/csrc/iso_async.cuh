// iso_async.cuh -- per-thread asynchronous global -> shared copies (cp.async),
// used to stage streamed values and histogram bins ahead of their use.
#pragma once
#include <cstdint>

// 16 bytes from global src to shared dst (a shared-window address), L2 only.
// src_bytes < 16 reads that many bytes and zero-fills the rest (0: no read).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes = 16u)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// Closes the thread's current group of copies.
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Waits until at most N of the thread's groups are still in flight; the copies
// of the older groups are then visible to this thread.
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ uint32_t shared_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
