// mirror_tables.h -- the occupancy terms of the mirror-boundary normal, shared
// by the host builder (geometry.cc) and the device builder (k_geom.cu).
//
// Each term is {neighbour slot, weight kind (1, 2 = 1/sqrt2, 3 = 1/sqrt3),
// sign}, in the reference's source order (GPU3D.cu:1569-1573 in 3D,
// new_11.cu:1586-1588 in 2D): the order of the FP64 sums decides last-bit
// ties in the nearest-voxel search, so both builders add the terms in this
// order.  3D slots 1..26 enumerate (dx, dy, dz) in x-, then y-, then z-major
// order skipping the centre (GPU3D.cu:1492-1544); 2D slots
// | 1 2 3 | 4 s 5 | 6 7 8 | have x to the right and y down
// (new_11.cu:1544-1565).
#pragma once

#define LQT_MIRROR_IC3                                                                                    \
    {{3, 3, 1},  {1, 3, -1},  {6, 2, 1},   {9, 3, 1},   {7, 3, -1},  {4, 2, -1},                             \
     {12, 2, 1}, {10, 2, -1}, {14, 1, 1},  {17, 2, 1},  {15, 2, -1}, {13, 1, -1},                            \
     {20, 3, 1}, {18, 3, -1}, {23, 2, 1},  {26, 3, 1},  {24, 3, -1}, {21, 2, -1}}
#define LQT_MIRROR_IR3                                                                                    \
    {{9, 3, 1},  {2, 2, -1},  {3, 3, -1},  {1, 3, -1},  {8, 2, 1},   {7, 3, 1},                              \
     {17, 2, 1}, {11, 1, -1}, {12, 2, -1}, {10, 2, -1}, {16, 1, 1},  {15, 2, 1},                             \
     {26, 3, 1}, {19, 2, -1}, {20, 3, -1}, {18, 3, -1}, {25, 2, 1},  {24, 3, 1}}
#define LQT_MIRROR_IL3                                                                                    \
    {{18, 3, 1}, {19, 2, 1},  {20, 3, 1},  {21, 2, 1},  {22, 1, 1},  {23, 2, 1},                             \
     {24, 3, 1}, {25, 2, 1},  {26, 3, 1},  {1, 3, -1},  {2, 2, -1},  {3, 3, -1},                             \
     {4, 2, -1}, {5, 1, -1},  {6, 2, -1},  {7, 3, -1},  {8, 2, -1},  {9, 3, -1}}
#define LQT_MIRROR_IL2 {{1, 2, -1}, {3, 2, 1}, {4, 1, -1}, {5, 1, 1}, {6, 2, -1}, {8, 2, 1}}
#define LQT_MIRROR_IR2 {{1, 2, -1}, {2, 1, -1}, {3, 2, -1}, {6, 2, 1}, {7, 1, 1}, {8, 2, 1}}
#define LQT_MIRROR_SLOT2X {0, -1, 0, 1, -1, 1, -1, 0, 1}
#define LQT_MIRROR_SLOT2Y {0, -1, -1, -1, 0, 0, 1, 1, 1}
