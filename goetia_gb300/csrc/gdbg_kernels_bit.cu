// Kernels and launchers for the bit storage.
#include "gdbg_launch_impl.cuh"

namespace gdbg {
GDBG_INSTANTIATE_LAUNCHERS(GDBG_BIT)
}  // namespace gdbg
