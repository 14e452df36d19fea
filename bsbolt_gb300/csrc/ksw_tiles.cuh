// ksw_tiles.cuh -- the tile shapes of the batched extension and the map that
// assigns one to every query length.
//
// A tile is G lanes per job (32/G jobs per warp) x C query columns per lane;
// it holds queries of up to G*C - 1 bases (columns 0..qlen).  Every shape in
// kTileList is compiled (ksw_tiles_g*.cu); a tile map picks, for each
// need = qlen + 1, the shape its jobs run on.  The default map below was
// chosen by timing every candidate shape per query-length band on a GB300;
// bsb_set_tile_map installs another one (e.g. the autotuner's) per context.
// The shape never changes a result, only the time.
#pragma once

#include "bsb_internal.cuh"

struct KswTile {
    int G, C;
};

constexpr KswTile kTileList[] = {
    {4, 1},   {4, 2},   {4, 3},   {4, 4},   {4, 5},   {4, 6},   {4, 7},   {4, 8},      //  0..7
    {4, 9},   {4, 10},  {4, 11},  {4, 12},  {4, 13},  {4, 14},  {4, 15},  {4, 16},     //  8..15
    {8, 6},   {8, 7},   {8, 8},   {8, 9},   {8, 10},  {8, 11},  {8, 12},  {8, 13},     // 16..23
    {8, 14},  {8, 15},  {8, 16},  {8, 17},  {8, 18},                                    // 24..28
    {16, 5},  {16, 6},  {16, 7},  {16, 8},  {16, 9},  {16, 10}, {16, 11}, {16, 12},    // 29..36
    {16, 13}, {16, 14}, {16, 15}, {16, 16},                                             // 37..40
    {32, 5},  {32, 6},  {32, 7},  {32, 8},  {32, 9},  {32, 10}, {32, 11}, {32, 12},    // 41..48
    {32, 13}, {32, 14}, {32, 15}, {32, 16},                                             // 49..52
    {32, 20}, {32, 24}, {32, 28}, {32, 32},                                             // 53..56
    {4, 20},  {4, 24},  {4, 28},  {4, 32}};                                             // 57..60
constexpr int kNumTiles = sizeof(kTileList) / sizeof(kTileList[0]);
constexpr int kMaxNeed = BSB_TILE_MAP_LEN - 1;    // columns 0..qlen with qlen <= 1023
constexpr int kKswBlock = 128;                      // threads per block (4 warps)

static_assert(kNumTiles == BSB_NUM_TILES, "tile list and public header disagree");
static_assert(kNumTiles <= 64, "tile sets are 64-bit masks");

// Shapes with a 16-bit two-columns-per-register kernel: an even C (every shape has C <= 32:
// a lane's non-zero columns are one 32-bit mask, and the 16-bit row-maximum key keeps a
// column index in 4 bits per half).
constexpr bool tile_has_pack16(int C) { return C % 2 == 0 && C <= 32; }

constexpr int tile_index(int G, int C)
{
    for (int t = 0; t < kNumTiles; ++t)
        if (kTileList[t].G == G && kTileList[t].C == C) return t;
    return -1;
}

struct KswTileMap {
    uint8_t tile[kMaxNeed + 1];    // [0] unused
};

// 4 lanes up to 128 columns (even C up to 16, then 20, 24, 28, 32), 8 lanes up to
// 144, 16 up to 256, then 32; the narrowest even C that holds the query within each
// group size (even C runs on 16-bit cells, two per register: cheaper than the
// next-narrower odd C).  Measured on GB300 with the autotuner on the 4M-job
// distribution: 4x20..4x32 beat 8x10..8x16 by 1.11-1.23x on the bands they hold (fewer
// lanes per job amortise a row's fixed work over more columns).
constexpr int even_up(int c) { return c + (c & 1); }
constexpr KswTileMap make_default_tile_map()
{
    KswTileMap m{};
    for (int need = 1; need <= kMaxNeed; ++need) {
        int t = 0;
        if (need <= 64) t = tile_index(4, even_up((need + 3) / 4));
        else if (need <= 128) t = tile_index(4, ((need + 15) / 16) * 4);
        else if (need <= 144) t = tile_index(8, even_up((need + 7) / 8 < 9 ? 9 : (need + 7) / 8));
        else if (need <= 256) t = tile_index(16, even_up((need + 15) / 16 < 10 ? 10 : (need + 15) / 16));
        else if (need <= 512) t = tile_index(32, even_up((need + 31) / 32 < 9 ? 9 : (need + 31) / 32));
        else if (need <= 640) t = tile_index(32, 20);
        else if (need <= 768) t = tile_index(32, 24);
        else if (need <= 896) t = tile_index(32, 28);
        else t = tile_index(32, 32);
        m.tile[need] = (uint8_t)t;
    }
    return m;
}

constexpr KswTileMap kDefaultTileMap = make_default_tile_map();

// Launches the persistent kernel of one tile shape over a range of the scheduled
// order: the jobs order[range[0] .. range[1]), drawn through *counter.
typedef cudaError_t (*KswTileLaunch)(const KswParams &P, const bsb_ext_job_t *jobs, const uint8_t *seq,
                                     const int32_t *order, const int32_t *range, int *counter,
                                     bsb_ext_out_t *out, int64_t *cells, int n_sm, cudaStream_t st);

KswTileLaunch ksw_tiles_g4(int C);
KswTileLaunch ksw_tiles_g8(int C);
KswTileLaunch ksw_tiles_g16(int C);
KswTileLaunch ksw_tiles_g32(int C);
KswTileLaunch ksw_tiles16_g4(int C);
KswTileLaunch ksw_tiles16_g8(int C);
KswTileLaunch ksw_tiles16_g16(int C);
KswTileLaunch ksw_tiles16_g32(int C);

// The 32-bit cell kernel of tile t (every shape has one).
inline KswTileLaunch ksw_tile_launcher(int t)
{
    if (t < 0 || t >= kNumTiles) return nullptr;
    const KswTile s = kTileList[t];
    switch (s.G) {
    case 4: return ksw_tiles_g4(s.C);
    case 8: return ksw_tiles_g8(s.C);
    case 16: return ksw_tiles_g16(s.C);
    case 32: return ksw_tiles_g32(s.C);
    default: return nullptr;
    }
}

// The 16-bit two-columns-per-register kernel of tile t (tile_has_pack16), or NULL.
inline KswTileLaunch ksw_tile16_launcher(int t)
{
    if (t < 0 || t >= kNumTiles || !tile_has_pack16(kTileList[t].C)) return nullptr;
    const KswTile s = kTileList[t];
    switch (s.G) {
    case 4: return ksw_tiles16_g4(s.C);
    case 8: return ksw_tiles16_g8(s.C);
    case 16: return ksw_tiles16_g16(s.C);
    case 32: return ksw_tiles16_g32(s.C);
    default: return nullptr;
    }
}
