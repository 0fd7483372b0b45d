// Grid kernel instantiation for 24 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(24)
