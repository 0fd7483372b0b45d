// Grid kernel instantiation for 4 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(4)
