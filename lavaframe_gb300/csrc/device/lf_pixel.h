// Order in which the paths of one sample of a tile visit its pixels (engine and per-batch
// path starts, and host readbacks of per-path results).
#pragma once

namespace lfd
{
// Pixel of the lp-th path of a sample in a visible tile of w x h: 8 x 4 blocks, in row-major
// block order, over the part of the tile that whole blocks cover, then the columns right of
// it and the rows below it, each row-major. A warp's 32 consecutive ids then trace an 8 x 4
// patch of camera rays instead of a 32 x 1 strip. Every pixel is taken once per sample.
__host__ __device__ inline void pixel_of(int lp, int w, int h, int& x, int& y)
{
    const int w8 = w & ~7, h4 = h & ~3;
    const int full = w8 * h4;
    if (lp < full)
    {
        const int blk = lp >> 5, j = lp & 31, bw = w8 >> 3;
        const int by = blk / bw;
        x = (blk - by * bw) * 8 + (j & 7);
        y = by * 4 + (j >> 3);
        return;
    }
    int r = lp - full;
    const int wr = w - w8;
    if (r < wr * h4)
    {
        y = r / wr;
        x = w8 + (r - y * wr);
        return;
    }
    r -= wr * h4;
    const int dy = r / w;
    y = h4 + dy;
    x = r - dy * w;
}
}
