#include "launch_impl.cuh"
namespace fg {
FG_INSTANTIATE(0, 1)
}
