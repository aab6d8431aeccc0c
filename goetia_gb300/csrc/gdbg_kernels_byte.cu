// Kernels and launchers for the byte storage.
#include "gdbg_launch_impl.cuh"

namespace gdbg {
GDBG_INSTANTIATE_LAUNCHERS(GDBG_BYTE)
}  // namespace gdbg
