// The faces a sweep tile solves.
//
// A face flux is read only by the update of a fluid cell beside it (the
// update, like the reference's, touches interior cells of type 0 only:
// MUSCL_Scheme.cpp:83,145): the X face (i+1/2, j) by cells (i, j) and
// (i+1, j), the Y face (i, j+1/2) by (i, j) and (i, j+1).  A tile that
// straddles a wall therefore solves only the faces with a fluid cell on one
// side, taken from a compacted list so that every warp works on faces that
// are needed.  The one other reader is the reference's Y-face slot reuse: a Y
// face (i, j-1/2) that keeps the X-face flux of its slot reads the X face
// (i+1/2, j-1), which the sweep solves after the Y faces where the list left
// it out (x_face_listed).
//
// Indexing, tile-local: the flag plane covers cells (i0-1 .. i0+TX,
// j0-1 .. j0+TY) as fluid[ly][lx] with lx = i - (i0-1), ly = j - (j0-1); the
// X faces of tile row r (sF row r+1) and the Y faces (sG rows 0..TY) are the
// candidates q < NXF and NXF <= q < NXF + NYF, in the sweep's own order.
#pragma once

#include <cstdint>

#include "internal.h"

namespace ibtfo {

template <int TX, int TY>
struct TileFaces
{
    static constexpr int NXF = (TX + 1) * TY; // X faces of the tile's rows
    static constexpr int NYF = TX * (TY + 1); // Y faces below, inside and above the tile
    unsigned char fluid[TY + 2][TX + 2];      // 1: an interior fluid cell (updated by the sweep)
    unsigned short list[NXF + NYF];           // the candidates some fluid cell reads
    int n;                                    // list length
    int all;                                  // every cell of the flag plane is fluid: the list is 0..NXF+NYF-1
                                              // (the flags are then not read)
};

// X face (i + 1/2, j) of candidate q < NXF: sF row r (1..TY), column fc (0..TX),
// between cells i0 + fc - 1 and i0 + fc of row j0 + r - 1
template <int TX, int TY>
__device__ __forceinline__ void x_face_of(int q, int &r, int &fc)
{
    if (q < TX * TY)
        r = q / TX + 1, fc = q - (r - 1) * TX; // a warp reads one row of the staged tile
    else
        r = q - TX * TY + 1, fc = TX; // the last column of each row after the others
}

// Y face of candidate q >= NXF: sG row r (0..TY), column c (0..TX-1),
// between cells (i0 + c, j0 + r - 1) and (i0 + c, j0 + r)
template <int TX, int TY>
__device__ __forceinline__ void y_face_of(int q, int &r, int &c)
{
    const int qq = q - TileFaces<TX, TY>::NXF;
    r = qq / TX;
    c = qq - r * TX;
}

// Flags of the tile's cells and their one-cell ring, and the list of the
// faces to solve (for a tile the list marks interior: `all`, no flags
// staged).  sKeep (the Y-face slot-reuse bits) is cleared for the Y faces
// left out, so that nothing reads a stale bit.  All NT threads call it;
// ends with a barrier.
template <int TX, int TY, int NT>
__device__ __forceinline__ void tile_faces_build(TileFaces<TX, TY> &f, unsigned char (*keep)[TX],
                                                 const GridDesc &g, const uint8_t *__restrict__ type, int i0,
                                                 int j0, bool interior = false)
{
    constexpr int W = TX + 2, H = TY + 2;
    constexpr int NC = TileFaces<TX, TY>::NXF + TileFaces<TX, TY>::NYF;
    const int tid = threadIdx.x;
    if (interior)
    {
        // the tile list marks the tile: every cell and its ring is fluid
        if (tid == 0)
        {
            f.n = NC;
            f.all = 1;
        }
        __syncthreads();
        return;
    }
    int mine = 1;
    for (int q = tid; q < W * H; q += NT)
    {
        const int ly = q / W, lx = q - ly * W;
        const int i = i0 - 1 + lx, j = j0 - 1 + ly;
        const bool in = i >= g.ng && i < g.ng + g.n_x && j >= g.ng && j < g.ng + g.n_y;
        const int fl = in && type[(long long)j * g.pitch + i] == 0;
        f.fluid[ly][lx] = (unsigned char)fl;
        mine &= fl;
    }
    if (tid == 0)
        f.n = 0;
    const int all = __syncthreads_and(mine);
    if (all)
    {
        if (tid == 0)
        {
            f.n = NC;
            f.all = 1;
        }
        __syncthreads();
        return;
    }
    const int lane = tid & 31;
    // a uniform trip count: every lane of every warp takes part in each ballot
    for (int base = 0; base < NC; base += NT)
    {
        const int q = base + tid;
        bool need = false;
        if (q < TileFaces<TX, TY>::NXF)
        {
            int r, fc;
            x_face_of<TX, TY>(q, r, fc);
            need = f.fluid[r][fc] | f.fluid[r][fc + 1];
        }
        else if (q < NC)
        {
            int r, c;
            y_face_of<TX, TY>(q, r, c);
            need = f.fluid[r][c + 1] | f.fluid[r + 1][c + 1];
            if (!need)
                keep[r][c] = 0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, need);
        int off = 0;
        if (lane == 0 && m)
            off = atomicAdd(&f.n, __popc(m));
        off = __shfl_sync(0xffffffffu, off, 0);
        if (need)
            f.list[off + __popc(m & ((1u << lane) - 1u))] = (unsigned short)q;
    }
    if (tid == 0)
        f.all = 0;
    __syncthreads();
}

// whether cell (tile-local column c, row r) is updated
template <int TX, int TY>
__device__ __forceinline__ bool tile_cell_fluid(const TileFaces<TX, TY> &f, int r, int c)
{
    return f.all || f.fluid[r + 1][c + 1];
}

// candidate of list position t
template <int TX, int TY>
__device__ __forceinline__ int tile_face(const TileFaces<TX, TY> &f, int t)
{
    return f.all ? t : (int)f.list[t];
}

// Whether the X face in sF row r, column fc was solved from the list (rows
// 1..TY; row 0, below the tile, never is).
template <int TX, int TY>
__device__ __forceinline__ bool x_face_listed(const TileFaces<TX, TY> &f, int r, int fc)
{
    return r > 0 && (f.all || f.fluid[r][fc] || f.fluid[r][fc + 1]);
}

} // namespace ibtfo
