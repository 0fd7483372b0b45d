// Table-screen kernel instantiation for 32 columns per lane.
#include "dto_table.cuh"
DTO_DEFINE_TABLE_GRID(32)
