// Table-screen kernel instantiation for 24 columns per lane.
#include "dto_table.cuh"
DTO_DEFINE_TABLE_GRID(24)
