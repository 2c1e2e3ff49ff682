// Path kernel instantiation unit (see kernels.cuh).
#include "kernels.cuh"

namespace nedev {

NE_PATH_KERNEL_INSTANCE(, 0, K_GENERAL | K_COUNT)
NE_PATH_KERNEL_INSTANCE(, 1, K_GENERAL | K_COUNT)
NE_PATH_KERNEL_INSTANCE(, 2, K_GENERAL | K_COUNT)

}  // namespace nedev
