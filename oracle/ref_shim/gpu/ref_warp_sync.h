/* TEST INFRASTRUCTURE ONLY: forced include for building the reference's
 * GPU/dyhash/cuckoo.cu for sm_103a.
 *
 * The reference was written for sm_61 and calls the pre-Volta warp
 * intrinsics __ballot(p) and __shfl(v, lane, width), which no longer exist.
 * Each of its kernels runs a 16-lane group per key (ELEM_NUM_P = 4), and the
 * two groups of a warp part ways at their `continue` statements
 * (cuckoo.cu:489, :554), so the replacement must name only the calling
 * lane's own group: lanes 0-15 or 16-31. Every lane of a group works on the
 * same key and reaches each intrinsic together, which is what the _sync
 * forms require.
 */
#pragma once
#include <cuda_runtime.h>

#define DYC_REF_GROUP_MASK (0xFFFFu << (threadIdx.x & 16u))
#define __ballot(p) __ballot_sync(DYC_REF_GROUP_MASK, (p))
#define __shfl(v, lane, width) __shfl_sync(DYC_REF_GROUP_MASK, (v), (lane), (width))
