// Path kernel instantiation unit (see kernels.cuh).
#include "kernels.cuh"

namespace nedev {

NE_PATH_KERNEL_INSTANCE(, 2, K_MESH)

}  // namespace nedev
