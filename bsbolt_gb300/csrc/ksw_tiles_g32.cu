// ksw_tiles_g32.cu -- extension kernels with 32 lanes (a warp) per job, 32-bit cells (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles_g32(int C)
{
    switch (C) {
    case 5: return ksw_tile_launch<5, 32>;
    case 6: return ksw_tile_launch<6, 32>;
    case 7: return ksw_tile_launch<7, 32>;
    case 8: return ksw_tile_launch<8, 32>;
    case 9: return ksw_tile_launch<9, 32>;
    case 10: return ksw_tile_launch<10, 32>;
    case 11: return ksw_tile_launch<11, 32>;
    case 12: return ksw_tile_launch<12, 32>;
    case 13: return ksw_tile_launch<13, 32>;
    case 14: return ksw_tile_launch<14, 32>;
    case 15: return ksw_tile_launch<15, 32>;
    case 16: return ksw_tile_launch<16, 32>;
    case 20: return ksw_tile_launch<20, 32>;
    case 24: return ksw_tile_launch<24, 32>;
    case 28: return ksw_tile_launch<28, 32>;
    case 32: return ksw_tile_launch<32, 32>;
    default: return nullptr;
    }
}
