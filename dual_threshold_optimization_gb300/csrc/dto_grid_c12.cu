// Grid kernel instantiation for 12 columns per lane.
#include "dto_grid.cuh"
DTO_DEFINE_GRID(12)
