// devpool.h -- the library's device memory: one stream-ordered CUDA memory
// pool per GPU, shared by the render path and the batch plans.
#pragma once
#include <cstddef>

#include <cuda_runtime.h>

namespace sonar {

// A block of at least `bytes` (1 if 0) ordered on stream s: work queued on s
// after this call may use it; another stream may use it once it has
// synchronised with s.  On cudaErrorMemoryAllocation the pool waits for the
// device, returns the memory it holds unused and tries once more.
cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t s);

// Returns p (may be null) to the pool once the work queued on s so far is
// done.  Nothing synchronises: the pool hands the block to a later
// allocation on s at once, and to one on another stream only after the
// stream-ordered dependency is met.
void pool_free(void *p, cudaStream_t s);

// Bytes of unused memory each pool keeps at a synchronisation point (what
// it holds above this is given back to the device then).
void pool_set_cache_limit(unsigned long long bytes);
unsigned long long pool_cache_limit();

// Waits for the device and gives every pool's unused memory back.
cudaError_t pool_trim();

// Bytes the current device's pool has mapped (in use + cached), or 0.
unsigned long long pool_reserved_bytes();

// Copies between pageable host memory and the device through two pinned
// chunks that live for the process, so the DMA runs at the link's rate while
// the host fills or drains the other chunk.  Copies below 256 KB go straight
// from pageable memory.
//
// stage_to_device returns once src has been read (src may be freed or
// reused); the copy into dst is ordered on s.
cudaError_t stage_to_device(void *dst, const void *src, size_t bytes, cudaStream_t s);
// stage_to_host returns once dst holds the data (s has reached the copy).
cudaError_t stage_to_host(void *dst, const void *src, size_t bytes, cudaStream_t s);

// Pinned host memory for arrays that are built on the host and copied to
// the device, kept for the process and grown on demand: writing them there
// costs no page faults and their copies run as plain DMA.  A region stays
// valid until host_arena_reset, which the caller makes only once every copy
// out of the arena is done.  host_arena_take returns null when no pinned
// memory can be had (the caller then builds the array in pageable memory).
void *host_arena_take(size_t bytes);
void host_arena_reset();

}  // namespace sonar
