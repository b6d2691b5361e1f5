#include "launch_z2_impl.cuh"
namespace fg {
FG_INSTANTIATE_Z2(1)
}
