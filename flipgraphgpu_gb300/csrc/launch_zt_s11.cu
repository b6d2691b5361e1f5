#include "launch_impl.cuh"
namespace fg {
FG_INSTANTIATE(1, 11)
}
