// Grid kernel instantiation for 8 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(8)
