// ksw_tiles_g16.cu -- extension kernels with 16 lanes per job, 32-bit cells (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles_g16(int C)
{
    switch (C) {
    case 5: return ksw_tile_launch<5, 16>;
    case 6: return ksw_tile_launch<6, 16>;
    case 7: return ksw_tile_launch<7, 16>;
    case 8: return ksw_tile_launch<8, 16>;
    case 9: return ksw_tile_launch<9, 16>;
    case 10: return ksw_tile_launch<10, 16>;
    case 11: return ksw_tile_launch<11, 16>;
    case 12: return ksw_tile_launch<12, 16>;
    case 13: return ksw_tile_launch<13, 16>;
    case 14: return ksw_tile_launch<14, 16>;
    case 15: return ksw_tile_launch<15, 16>;
    case 16: return ksw_tile_launch<16, 16>;
    default: return nullptr;
    }
}
