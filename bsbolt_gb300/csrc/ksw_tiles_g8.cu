// ksw_tiles_g8.cu -- extension kernels with 8 lanes per job, 32-bit cells (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles_g8(int C)
{
    switch (C) {
    case 6: return ksw_tile_launch<6, 8>;
    case 7: return ksw_tile_launch<7, 8>;
    case 8: return ksw_tile_launch<8, 8>;
    case 9: return ksw_tile_launch<9, 8>;
    case 10: return ksw_tile_launch<10, 8>;
    case 11: return ksw_tile_launch<11, 8>;
    case 12: return ksw_tile_launch<12, 8>;
    case 13: return ksw_tile_launch<13, 8>;
    case 14: return ksw_tile_launch<14, 8>;
    case 15: return ksw_tile_launch<15, 8>;
    case 16: return ksw_tile_launch<16, 8>;
    case 17: return ksw_tile_launch<17, 8>;
    case 18: return ksw_tile_launch<18, 8>;
    default: return nullptr;
    }
}
