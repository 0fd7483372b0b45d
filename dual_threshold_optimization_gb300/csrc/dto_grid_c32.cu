// Grid kernel instantiation for 32 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(32)
