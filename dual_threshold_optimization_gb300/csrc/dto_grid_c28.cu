// Grid kernel instantiation for 28 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(28)
