// ksw_tiles_g4.cu -- extension kernels with 4 lanes per job, 32-bit cells (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles_g4(int C)
{
    switch (C) {
    case 1: return ksw_tile_launch<1, 4>;
    case 2: return ksw_tile_launch<2, 4>;
    case 3: return ksw_tile_launch<3, 4>;
    case 4: return ksw_tile_launch<4, 4>;
    case 5: return ksw_tile_launch<5, 4>;
    case 6: return ksw_tile_launch<6, 4>;
    case 7: return ksw_tile_launch<7, 4>;
    case 8: return ksw_tile_launch<8, 4>;
    case 9: return ksw_tile_launch<9, 4>;
    case 10: return ksw_tile_launch<10, 4>;
    case 11: return ksw_tile_launch<11, 4>;
    case 12: return ksw_tile_launch<12, 4>;
    case 13: return ksw_tile_launch<13, 4>;
    case 14: return ksw_tile_launch<14, 4>;
    case 15: return ksw_tile_launch<15, 4>;
    case 16: return ksw_tile_launch<16, 4>;
    case 20: return ksw_tile_launch<20, 4>;
    case 24: return ksw_tile_launch<24, 4>;
    case 28: return ksw_tile_launch<28, 4>;
    case 32: return ksw_tile_launch<32, 4>;
    default: return nullptr;
    }
}
