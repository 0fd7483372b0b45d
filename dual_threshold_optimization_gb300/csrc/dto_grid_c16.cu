// Grid kernel instantiation for 16 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(16)
