// Tables of the tensor-core polynomial evaluation (generated by
// codegen/gen_poly_tc.py into the build folder; see poly_tc.cu).
#pragma once

namespace mbpol {

struct PolyTCTables {
    int nv;     // variables
    int ny;     // rows of the quadratic form: 1 + nv + nv (nv + 1) / 2
    int npad;   // ny rounded up to 16
    int nrt;    // row tiles in the warp lists
    int nent;   // kept 16x16 tiles
    const float* x0h;              // expansion point, hi and lo parts [nv]
    const float* x0l;
    const float* inv_bound;        // [nv]: 1 / (sampled maximum of |x - x0|)
    const unsigned* ymeta;         // [npad]: a | b << 8 | (s + 128) << 16; y = d_a d_b 2^s with
                                   // d_nv = 1 and d_{nv+1} = 0
    const float* rowscale;         // [npad]: 2^-r_m (0 for padding rows)
    const int* warp_begin;         // [9]: row tiles of warp w: rt_id[warp_begin[w] .. warp_begin[w+1])
    const int* rt_id;              // [nrt]
    const int* rt_entry;           // [nrt + 1]: tiles of row tile i: ent_kt[rt_entry[i] .. rt_entry[i+1])
    const unsigned short* ent_kt;  // [nent]: k-tile of each kept tile
    const unsigned* frag;          // [nent][3 pieces][32 lanes][4 registers]: fp16 pairs
    // tcgen05 kernel (poly_tc5.cu): S as a stream of blocks of `rows5` rows x
    // 16 columns, ordered by K part, row chunk, k-tile
    int parts5;                    // K parts (Y' of one part in tensor memory)
    int rows5;                     // rows of S per chunk (N of the MMA)
    int nblk5;                     // blocks in the stream
    const unsigned short* sblk;    // [nblk5][3 pieces][2 k halves][rows5 / 8][8 rows][8 k]: fp16
    const unsigned char* blk_kt;   // [nblk5]: k-tile of each block within its part
    const int* blk_begin;          // [parts5 * npad / rows5 + 1]: first block of (part, chunk)
};

extern const PolyTCTables k_poly2b;
extern const PolyTCTables k_poly3b;

}  // namespace mbpol
