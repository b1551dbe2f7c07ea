// Internal definitions shared by the GB300 Z-grid kernels.
//
// Data layout in HBM (one "arena" per batch of segments; a plain tay_run is a batch of
// one segment):
//   * agents of all segments are concatenated; segment s owns [begin, begin + count);
//   * every agent field lives in a structure-of-arrays stream: float4 streams (16 B per
//     agent, coalesced 16-byte loads) and u32 streams;
//   * state streams are double-buffered ("cur" / "alt"): the sort gathers them into
//     cell order, a fused see+act pass writes the fields it changes into the other copy;
//   * per-step streams (accumulators, density/pressure) are single-buffered and valid
//     only inside one step;
//   * a cell table per segment: Morton order, uint2 {first, end} per cell, written only
//     at non-empty cells; row order, one header per (y, z) row {x_first, x_last, first,
//     end} plus start entries over each row's occupied span.  Written after each sort and
//     cleared the same way before the next one (the reference clears its table per step
//     too, tay/cpu_z_grid.c:223-225);
//   * per segment and step, the grid (origin, cell size, cells per axis) and its rounding
//     pad, derived once from the bounding box.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define TGPU_HD __host__ __device__ __forceinline__
#define TGPU_D __device__ __forceinline__

namespace tgpu {

constexpr int kMaxF4 = 8;   // float4 streams per model
constexpr int kMaxU32 = 2;  // u32 streams per model
constexpr int kSortTile = 2048;       // agents per radix tile (256 threads x 8)
constexpr int kSortThreads = 256;
constexpr int kSeeThreads = 128;      // seers per see CTA

// Static per-segment description, written by the host once per run.
struct SegmentSpec {
    uint32_t begin;          // first agent (index into the concatenated streams)
    uint32_t count;          // agents in this segment
    uint32_t table_base;     // first entry of this segment's dense cell table
    uint32_t table_cap;      // entries available to it
    uint32_t tile_begin;     // first radix tile of this segment
    uint32_t tile_count;     // radix tiles of this segment
    uint32_t axis_cells_max; // power of two, <= 1024: bounds each grid axis (key bits)
    uint32_t fixed_box;      // 1: use box_min/box_max instead of the agents' bounding box
    uint32_t order;          // cell order of the keys and table layout: kOrderMorton / kOrderRows
    uint32_t dims;           // tay_configure_space dims (1..3; 0 means 3): axes >= dims get one cell
    uint32_t row_cap;        // row order: (y, z) rows the table's header region holds
    uint32_t axis_cells_y;   // row order: power-of-two bounds of the y and z axes (x: axis_cells_max)
    uint32_t axis_cells_z;
    float part[3];           // minimum cell edge per axis
    float reach[3];          // largest see radius per axis over the segment's see passes
    float box_min[3];        // fixed space box (tay_fix_space_box)
    float box_max[3];
};

// Per-step grid, derived on the device from the bounding box.  Every kernel derives
// it with the same function from the same inputs, so all kernels agree bit for bit.
struct Grid {
    float origin[3];
    float inv_cs[3];
    float cs[3];
    int dims[3];
};

// Bounding box accumulator: order-preserving u32 encodings so that atomicMin/atomicMax
// on unsigned integers order floats correctly.
struct BoxAcc {
    uint32_t lo[3];
    uint32_t hi[3];
    uint32_t size[3];  // non-point agents: largest max - min per axis (ordered encoding)
};

TGPU_HD uint32_t float_to_ordered(float f) {
#ifdef __CUDA_ARCH__
    uint32_t b = __float_as_uint(f);
#else
    union { float f; uint32_t u; } cvt;
    cvt.f = f;
    uint32_t b = cvt.u;
#endif
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

TGPU_HD float ordered_to_float(uint32_t o) {
    uint32_t b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    union { float f; uint32_t u; } cvt;
    cvt.u = b;
    return cvt.f;
#endif
}

// Grid rule (GPU Z-grid): cells of edge >= part (the requested minimum part size, as in
// tay_configure_space), covering [min, max] of the box; each axis at most
// axis_cells_max cells and the whole grid at most table_cap cells, enlarging the cells
// when either bound would be exceeded (the reference shrinks its grid to its memory in
// the same spirit, tay/cpu_z_grid.c:175-176, tay/cpu_grid.c:95-106).
TGPU_HD int clamp_cells(float cells, uint32_t axis_max) {
    // NaN and values below 1 give one cell; never more than axis_max
    if (!(cells >= 1.0f)) return 1;
    if (cells > (float)axis_max) return (int)axis_max;
    return (int)cells;
}

TGPU_HD int seg_dims(const SegmentSpec &s) { return (s.dims >= 1u && s.dims <= 3u) ? (int)s.dims : 3; }

// Two cell orders.  kOrderMorton: the 3-D Morton key, a table entry {first, end} per
// cell.  kOrderRows: x fastest inside rows of constant (y, z), the rows in 2-D Morton
// order of (y, z): key = (row_code(y, z) << b) | x with b = log2(axis_cells_max), so the
// agents of x-adjacent cells are contiguous and a seer's box is one candidate range per
// row.  Its table holds, per row, a 16-byte header {x_first, x_last, first, end} (the
// occupied cells and the row's agent range; zero for an empty row) and, per cell x in
// (x_first, x_last], the first agent of the row in a cell >= x; entries outside that span
// are never read.  Both orders give the same neighbour sets; only the order in which a
// seer meets its neighbours differs.
enum CellOrder : uint32_t { kOrderMorton = 0, kOrderRows = 1 };

// Row-order table layout (u32 words from the segment's table base): the row headers
// (uint4, 16-byte aligned) at word 0 for up to row_cap rows, then the start entries at
// word 4 * row_cap + row * dims[0] + x.  The header region's place does not depend on the
// step's grid, so a header is never a stale entry of an earlier step: every step's clear
// leaves all headers zero.
TGPU_HD uint32_t row_entry_word(const SegmentSpec &s) { return 4u * s.row_cap; }

// Whether a grid fits the segment's table.
TGPU_HD bool table_fits(const SegmentSpec &s, const int *d) {
    const unsigned long long cells = (unsigned long long)d[0] * (unsigned long long)d[1] * (unsigned long long)d[2];
    if (s.order != kOrderRows) return cells <= s.table_cap;
    const unsigned long long rows = (unsigned long long)d[1] * (unsigned long long)d[2];
    return rows <= s.row_cap && 4ull * s.row_cap + cells <= 2ull * s.table_cap;
}

// Cell budget of axis i: in row order the x axis (whose cells only tighten each row's
// candidate range) and the y / z axes (whose cells make the rows) have their own bounds.
TGPU_HD uint32_t axis_max(const SegmentSpec &s, int i) {
    if (i > 0 && s.order == kOrderRows) {
        const uint32_t a = i == 1 ? s.axis_cells_y : s.axis_cells_z;
        if (a) return a;
    }
    return s.axis_cells_max;
}

TGPU_HD Grid derive_grid(const SegmentSpec &s, const float *mn, const float *mx) {
    Grid g;
    float cs[3], ext[3];
    int d[3];
    for (int i = 0; i < 3; ++i) {
        ext[i] = mx[i] - mn[i];
        if (!(ext[i] >= 0.0f) || ext[i] > 3.0e38f) ext[i] = 0.0f;
        cs[i] = s.part[i] > 0.0f ? s.part[i] : 1.0f;
        float cells = floorf(ext[i] / cs[i]) + 1.0f;
        if (cells > (float)axis_max(s, i)) cs[i] = ext[i] / ((float)axis_max(s, i) - 0.5f);
        d[i] = clamp_cells(floorf(ext[i] / cs[i]) + 1.0f, axis_max(s, i));
        if (i >= seg_dims(s)) {
            // an axis the space does not have: one cell spanning it
            d[i] = 1;
            cs[i] = ext[i] > cs[i] ? ext[i] : cs[i];
        }
    }
    for (int iter = 0; iter < 64; ++iter) {
        if (table_fits(s, d)) break;
        for (int i = 0; i < seg_dims(s); ++i) {
            cs[i] *= 1.25f;
            d[i] = clamp_cells(floorf(ext[i] / cs[i]) + 1.0f, axis_max(s, i));
        }
    }
    if (!table_fits(s, d)) {
        for (int i = 0; i < 3; ++i) {
            d[i] = 1;
            cs[i] = ext[i] > cs[i] ? ext[i] : cs[i];
        }
    }
    for (int i = 0; i < 3; ++i) {
        g.origin[i] = mn[i];
        g.cs[i] = cs[i];
        g.inv_cs[i] = 1.0f / cs[i];
        g.dims[i] = d[i];
    }
    return g;
}

TGPU_HD int cell_coord(float p, float origin, float inv_cs, int dim) {
    int c = (int)floorf((p - origin) * inv_cs);
    return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

// 3-D Morton code, 10 bits per axis, x at bit 0 (the reference's key layout,
// tay/cpu_z_grid.c:57-77, written here with the usual magic-number spread).
TGPU_HD uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

TGPU_HD uint32_t compact10(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0xFF0000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
}

TGPU_HD uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

// 2-D Morton spread / compaction of 10 bits (bit k to bit 2k).
TGPU_HD uint32_t spread2_10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

TGPU_HD uint32_t compact2_10(uint32_t v) {
    v &= 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0F0F0F0Fu;
    v = (v | (v >> 4)) & 0x00FF00FFu;
    v = (v | (v >> 8)) & 0x0000FFFFu;
    return v & 0x3FFu;
}


// log2 of a power-of-two bound of at most 1024 cells (0 for 0 or 1).
TGPU_HD uint32_t bound_bits(uint32_t v) {
#ifdef __CUDA_ARCH__
    return 31u - (uint32_t)__clz(v | 1u);
#else
    uint32_t b = 0;
    while ((2u << b) <= v && b < 10) ++b;
    return b;
#endif
}

TGPU_HD uint32_t axis_bits(const SegmentSpec &s) { return bound_bits(s.axis_cells_max); }

// Row order's code of row (y, z): a 2-D Morton code of the low min(by, bz) bits of both
// (by, bz: the bits of the y and z bounds), with the remaining high bits of the longer
// axis above it, so that the code takes by + bz bits and rows close in (y, z) are close
// in the order.
TGPU_HD uint32_t row_code(const SegmentSpec &s, uint32_t y, uint32_t z) {
    const uint32_t by = bound_bits(s.axis_cells_y), bz = bound_bits(s.axis_cells_z);
    const uint32_t m = by < bz ? by : bz;
    const uint32_t low = (1u << m) - 1u;
    const uint32_t code = spread2_10(y & low) | (spread2_10(z & low) << 1);
    return code | ((by > bz ? (y >> m) : (z >> m)) << (2u * m));
}

// The (y, z) of a row code.
TGPU_HD void row_of_code(const SegmentSpec &s, uint32_t code, uint32_t &y, uint32_t &z) {
    const uint32_t by = bound_bits(s.axis_cells_y), bz = bound_bits(s.axis_cells_z);
    const uint32_t m = by < bz ? by : bz;
    const uint32_t lo = code & ((1u << (2u * m)) - 1u), hi = code >> (2u * m);
    y = compact2_10(lo);
    z = compact2_10(lo >> 1);
    if (by > bz)
        y |= hi << m;
    else
        z |= hi << m;
}

TGPU_HD uint32_t cell_key(const SegmentSpec &s, uint32_t x, uint32_t y, uint32_t z) {
    if (s.order == kOrderRows) return (row_code(s, y, z) << axis_bits(s)) | x;
    return morton3(x, y, z);
}

// The step's grid of a segment: from its fixed box, or from the bounding box of its
// positions accumulated by the box kernel.
TGPU_HD Grid segment_grid(const SegmentSpec &s, const BoxAcc &b) {
    float mn[3], mx[3];
    for (int i = 0; i < 3; ++i) {
        mn[i] = s.fixed_box ? s.box_min[i] : ordered_to_float(b.lo[i]);
        mx[i] = s.fixed_box ? s.box_max[i] : ordered_to_float(b.hi[i]);
    }
    return derive_grid(s, mn, mx);
}

// Largest rounding error, in cells, of a cell coordinate computed as
// floor((p - origin) * inv_cs): a few ulps of the largest coordinate magnitude plus the
// relative error of the multiply on coordinates up to 1024 cells.
TGPU_D float grid_pad(const Grid &g, const SegmentSpec &s, const BoxAcc &b) {
    float m = 0.0f, csmin = g.cs[0];
    for (int a = 0; a < 3; ++a) {
        float lo = s.fixed_box ? s.box_min[a] : ordered_to_float(b.lo[a]);
        float hi = s.fixed_box ? s.box_max[a] : ordered_to_float(b.hi[a]);
        m = fmaxf(m, fmaxf(fabsf(lo), fabsf(hi)));
        csmin = fminf(csmin, g.cs[a]);
    }
    float ulp = m * 1.1920929e-7f;  // 2^-23
    return fmaxf(1.0f / 512.0f, 16.0f * ulp / csmin + 1024.0f * 4.0f * 1.1920929e-7f);
}

// A segment's grid for one step with its rounding pad (grid_pad), derived once per step
// from the bounding box by the grid kernel and read by every later kernel of the step.
struct SegGrid {
    Grid g;
    float pad;
};

// Device-side error word: kernels never trap; they record the first failure here and
// the host turns it into TAY_ERROR_CUDA.
enum DeviceError : uint32_t {
    kErrNone = 0,
    kErrTableOverflow = 1,
    kErrSortLookback = 2,  // a radix pass's look-back wait ran out (a tile never published)
    kErrStageWait = 4,     // a see CTA's wait for its bulk copies ran out
    kErrStageRange = 8,    // a lane's row range fell outside its row's staged run (skipped)
};

}  // namespace tgpu
