// pg_zobrist.cuh -- 128-bit Zobrist keys and the transposition-table entry
// format, shared by the device kernels (pg_tt.cu) and the host-side C ABI
// helpers that test them without a GPU.
//
// Keys follow the reference's HashKey128b (chess.h:410-452,
// computeZobristKey128b MoveGeneratorBitboard.h:3914-3980): two independent
// 64-bit Zobrist words per position.  Feature layout: 768 piece-square keys
// (6 piece kinds x 2 colours x 64 squares), 4 castling rights, 8 en-passant
// files, 1 side to move; the values are a fresh seeded set (splitmix64 from
// two seeds) rather than the reference's randoms.cpp -- counts never depend
// on the key values.
//
// Entry: 32 bytes (one DRAM sector), written as two 16-byte stores
//     e0 = k0 ^ v,  e1 = k1 ^ v,  e2 = v,  e3 = mix(k0, k1) ^ v
// and accepted for key k only when e0 ^ e2 == k0, e1 ^ e2 == k1 and
// e3 ^ e2 == mix(k0, k1).  The reference verifies the high word and the
// non-index bits of the low word of a 16-byte entry (perft_bb.h:690-693);
// here every key bit is compared, so an intact entry of another position
// is accepted only if its 128-bit key equals the probe's: with the slot
// taken from the low log2(entries) bits of k0, that is 2^-(128 - log2(entries))
// per probe of an occupied slot.  Two threads storing different positions
// into one slot at once can leave halves of two stores (the halves are not
// written as one transaction); such an entry is accepted for a key k only if
// the second half came from a store of k itself (then v is k's count) or if
// two independent 64-bit equalities hold by chance (about 2^-128).
#pragma once
#include <cuda_runtime.h>

#include "pg_types.h"

namespace pg {

constexpr int ZOBRIST_KEYS = 781;
constexpr int Z_CASTLE = 768, Z_EP = 772, Z_SIDE = 780;
constexpr u64 ZOBRIST_SEED0 = 0x5EED2B1D0C0FFEE5ull;
constexpr u64 ZOBRIST_SEED1 = 0xA24BAED4963EE407ull;

// the 781 key pairs: word x from the splitmix64 stream of seed 0, word y
// from the stream of seed 1
inline void zobrist_key_table(ulonglong2* out)
{
    u64 s0 = ZOBRIST_SEED0, s1 = ZOBRIST_SEED1;
    auto next = [](u64& s) {
        u64 z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int i = 0; i < ZOBRIST_KEYS; i++) {
        out[i].x = next(s0);
        out[i].y = next(s1);
    }
}

__host__ __device__ __forceinline__ int zb_lsb(u64 x)
{
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

// The 128-bit key of a board (48-byte HexaBitBoardPosition words: white,
// pawns + packed state, knights, bishop_queens, rook_queens, kings).  The
// half-move clock is not part of the key.  Never (0, 0): that is an empty
// table slot.
__host__ __device__ __forceinline__ ulonglong2 zobrist128(const u64* bw, const ulonglong2* z)
{
    const u64 w = bw[0], pawns = bw[1] & 0x00FFFFFFFFFFFF00ull, n = bw[2], bq = bw[3], rq = bw[4], k = bw[5];
    const u64 sets[6] = {pawns, n, bq & ~rq, rq & ~bq, bq & rq, k};
    u64 h0 = 0, h1 = 0;
#pragma unroll
    for (int t = 0; t < 6; t++) {
        for (u64 s = sets[t] & w; s; s &= s - 1) {
            const ulonglong2 e = z[t * 64 + zb_lsb(s)];
            h0 ^= e.x;
            h1 ^= e.y;
        }
        for (u64 s = sets[t] & ~w; s; s &= s - 1) {
            const ulonglong2 e = z[(6 + t) * 64 + zb_lsb(s)];
            h0 ^= e.x;
            h1 ^= e.y;
        }
    }
    const u64 st = bw[1];
    const int flags[4] = {(int)(st & 1), (int)((st >> 1) & 1), (int)((st >> 2) & 1), (int)((st >> 3) & 1)};
#pragma unroll
    for (int c = 0; c < 4; c++)
        if (flags[c]) {
            h0 ^= z[Z_CASTLE + c].x;
            h1 ^= z[Z_CASTLE + c].y;
        }
    const int ep = (int)((st >> 4) & 15);
    if (ep) {
        h0 ^= z[Z_EP + ((ep - 1) & 7)].x;
        h1 ^= z[Z_EP + ((ep - 1) & 7)].y;
    }
    if (st >> 63) {
        h0 ^= z[Z_SIDE].x;
        h1 ^= z[Z_SIDE].y;
    }
    if (!(h0 | h1)) h0 = 1;
    return make_ulonglong2(h0, h1);
}

// The key of board cw from the key kp of board pw: kp XOR the features in
// which the two boards differ.  For a parent and its child that is the
// squares the move changed (two to four), the castling rights it cleared,
// the old and new en-passant file and the side to move -- the update the
// reference applies while making a move (makeMove<c, true>,
// MoveGeneratorBitboard.h:3575-3836), taken here from the two boards instead
// of from the move.  XOR is linear over the feature sets, so the result
// equals zobrist128(cw) for any two boards; only the work depends on how
// many features differ.  A key (1, 0) may stand for the raw key 0 (the
// empty-slot remap above), so from such a key the board is keyed in full.
__host__ __device__ __forceinline__ ulonglong2 zobrist128_from(const u64* pw, ulonglong2 kp, const u64* cw,
                                                               const ulonglong2* z)
{
    if (kp.x == 1 && kp.y == 0) return zobrist128(cw, z);
    const u64 pp = pw[1] & 0x00FFFFFFFFFFFF00ull, cp = cw[1] & 0x00FFFFFFFFFFFF00ull;
    const u64 ps[6] = {pp, pw[2], pw[3] & ~pw[4], pw[4] & ~pw[3], pw[3] & pw[4], pw[5]};
    const u64 cs[6] = {cp, cw[2], cw[3] & ~cw[4], cw[4] & ~cw[3], cw[3] & cw[4], cw[5]};
    u64 h0 = kp.x, h1 = kp.y;
#pragma unroll
    for (int t = 0; t < 6; t++) {
        for (u64 s = (ps[t] & pw[0]) ^ (cs[t] & cw[0]); s; s &= s - 1) {
            const ulonglong2 e = z[t * 64 + zb_lsb(s)];
            h0 ^= e.x;
            h1 ^= e.y;
        }
        for (u64 s = (ps[t] & ~pw[0]) ^ (cs[t] & ~cw[0]); s; s &= s - 1) {
            const ulonglong2 e = z[(6 + t) * 64 + zb_lsb(s)];
            h0 ^= e.x;
            h1 ^= e.y;
        }
    }
    const u64 ds = pw[1] ^ cw[1];
#pragma unroll
    for (int c = 0; c < 4; c++)
        if ((ds >> c) & 1) {
            h0 ^= z[Z_CASTLE + c].x;
            h1 ^= z[Z_CASTLE + c].y;
        }
    const int pe = (int)((pw[1] >> 4) & 15), ce = (int)((cw[1] >> 4) & 15);
    if (pe) {
        h0 ^= z[Z_EP + ((pe - 1) & 7)].x;
        h1 ^= z[Z_EP + ((pe - 1) & 7)].y;
    }
    if (ce) {
        h0 ^= z[Z_EP + ((ce - 1) & 7)].x;
        h1 ^= z[Z_EP + ((ce - 1) & 7)].y;
    }
    if (ds >> 63) {
        h0 ^= z[Z_SIDE].x;
        h1 ^= z[Z_SIDE].y;
    }
    if (!(h0 | h1)) h0 = 1;
    return make_ulonglong2(h0, h1);
}

__host__ __device__ __forceinline__ u64 tt_mix(u64 k0, u64 k1) { return k0 ^ ((k1 << 29) | (k1 >> 35)); }

// entry words for key (k0, k1) and count v
__host__ __device__ __forceinline__ void tt_pack(u64 k0, u64 k1, u64 v, ulonglong2& a, ulonglong2& b)
{
    a = make_ulonglong2(k0 ^ v, k1 ^ v);
    b = make_ulonglong2(v, tt_mix(k0, k1) ^ v);
}

// true (and *v = the count) when the entry halves a, b hold key (k0, k1)
__host__ __device__ __forceinline__ bool tt_match(const ulonglong2& a, const ulonglong2& b, u64 k0, u64 k1, u64& v)
{
    v = b.x;
    return ((a.x ^ b.x) == k0) & ((a.y ^ b.x) == k1) & ((b.y ^ b.x) == tt_mix(k0, k1));
}

}  // namespace pg
