// Programmatic dependent launch inside the Arnoldi body.  A kernel launched with the
// programmatic stream-serialisation attribute is scheduled once every block of its
// predecessor has called pdl_trigger() (or exited), so its launch and its first loads
// overlap the predecessor's tail (at small meshes the tail is the last block's grid
// reduction and the Givens step).  Rules every body kernel keeps:
//   * pdl_wait() before the first read of anything its predecessor writes (the wait
//     returns once the predecessor has completed and its writes are visible);
//   * pdl_trigger() only after its own pdl_wait(), so a kernel that starts early finds
//     every kernel before its predecessor complete: its prologue may read their outputs.
// For a kernel launched without the attribute both are no-ops.
#pragma once

namespace cfdg {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace cfdg
