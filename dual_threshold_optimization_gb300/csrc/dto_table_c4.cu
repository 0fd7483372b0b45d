// Table-screen kernel instantiation for 4 columns per lane.
#include "dto_table.cuh"
DTO_DEFINE_TABLE_GRID(4)
