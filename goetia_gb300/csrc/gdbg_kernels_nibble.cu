// Kernels and launchers for the nibble storage.
#include "gdbg_launch_impl.cuh"

namespace gdbg {
GDBG_INSTANTIATE_LAUNCHERS(GDBG_NIBBLE)
}  // namespace gdbg
