// gather_core.cuh -- bicubic window sampling of a TMA-loaded screen tile.
// Host-compilable (__host__ __device__) so that the tile geometry can be
// checked by the CPU emulation against the oracle's per-pixel sampling.
#pragma once
#include "engine.cuh"

namespace atmwfs {

// Keys (a = -1/2) cubic convolution weights for taps at -1, 0, 1, 2.
AW_HD void keys_weights(float t, float w[4])
{
    const float t2 = t * t, t3 = t2 * t;
    w[0] = 0.5f * (-t3 + 2.0f * t2 - t);
    w[1] = 0.5f * (3.0f * t3 - 5.0f * t2 + 2.0f);
    w[2] = 0.5f * (-3.0f * t3 + 4.0f * t2 + t);
    w[3] = 0.5f * (t3 - t2);
}

struct TileGeom {
    int xs, ys, d;
    float fx, fy;
};

// Tile origin of layer position p for a CTA whose first row is y0, in the
// pass orientation (orient 1 exchanges the roles of the two screen axes).
AW_HD TileGeom tile_geom(LayerPos p, int orient, int y0)
{
    TileGeom g;
    const int ix = orient ? p.iy : p.ix;
    const int iy = orient ? p.ix : p.iy;
    g.fx = orient ? p.fy : p.fx;
    g.fy = orient ? p.fx : p.fy;
    g.xs = (ix + kPadX - 1) & ~3;
    g.d = ix + kPadX - 1 - g.xs;
    g.ys = iy + y0 + kPadY - 1;
    return g;
}

// Element (row r, column c) of a TMA tile made of NBOX boxes of kBoxW x TROWS.
template <int TROWS>
AW_HD int tile_index(int r, int c) { return ((c >> 5) * TROWS + r) * kBoxW + (c & (kBoxW - 1)); }

// Interpolate one layer for the CTA's RR rows.  Thread tid walks columns
// x = tid, tid + NT, ...; for each it forms the RR + 3 horizontal cubic
// sums of the tile rows and slides the vertical cubic down the column.
// Calls emit(r, x, value) for every pixel.
template <int N, int RR, int NT, typename F>
AW_HD void gather_tile(const float* tile, const TileGeom& g, float sc, int tid, F emit)
{
    constexpr int TROWS = RR + 3;
    float wx[4], wy[4];
    keys_weights(g.fx, wx);
    keys_weights(g.fy, wy);
    for (int x = tid; x < N; x += NT) {
        const int c = g.d + x;
        float h[TROWS];
        AW_UNROLL
        for (int b = 0; b < TROWS; b++) {
            h[b] = wx[0] * tile[tile_index<TROWS>(b, c)] + wx[1] * tile[tile_index<TROWS>(b, c + 1)] +
                   wx[2] * tile[tile_index<TROWS>(b, c + 2)] + wx[3] * tile[tile_index<TROWS>(b, c + 3)];
        }
        AW_UNROLL
        for (int r = 0; r < RR; r++) {
            const float val = (wy[0] * h[r] + wy[1] * h[r + 1] + wy[2] * h[r + 2] + wy[3] * h[r + 3]) * sc;
            emit(r, x, val);
        }
    }
}

}  // namespace atmwfs
