// Grid kernel instantiation for 20 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(20)
