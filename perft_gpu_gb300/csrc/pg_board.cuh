// pg_board.cuh -- board type, constants and bit primitives for the sm_103a
// move generator.
//
// The 48-byte board is the reference's HexaBitBoardPosition
// (chess.h:207-230): six 64-bit words, with the game state packed into the
// rank-1 and rank-8 bytes of the pawn word (castling bits 0-3, en-passant
// file+1 bits 4-7, half-move counter bits 56-62, side to move bit 63).
#pragma once
#include <cstdint>

#include "pg_types.h"

namespace pg {

struct Pos {
    u64 w;   // whitePieces
    u64 p;   // pawns (ranks 2-7) + packed state
    u64 n;   // knights
    u64 bq;  // bishops and queens
    u64 rq;  // rooks and queens
    u64 k;   // kings
};

constexpr u64 FILE_A = 0x0101010101010101ull;
constexpr u64 FILE_H = 0x8080808080808080ull;
constexpr u64 NOT_A = ~FILE_A;
constexpr u64 NOT_H = ~FILE_H;
constexpr u64 RANK_1 = 0x00000000000000FFull;
constexpr u64 RANK_3 = 0x0000000000FF0000ull;
constexpr u64 RANK_6 = 0x0000FF0000000000ull;
constexpr u64 RANK_8 = 0xFF00000000000000ull;
constexpr u64 BACK_RANKS = RANK_1 | RANK_8;
constexpr u64 INNER = 0x00FFFFFFFFFFFF00ull;
constexpr u64 DIAG_A1H8 = 0x8040201008040201ull;
constexpr u64 DIAG_A8H1 = 0x0102040810204080ull;

// castling square sets of the reference (MoveGeneratorBitboard.h:43-55)
constexpr u64 W_KS_PATH = 0x60ull;
constexpr u64 W_QS_SAFE = 0x0Cull;
constexpr u64 W_QS_PATH = 0x0Eull;
constexpr u64 B_KS_PATH = 0x6000000000000000ull;
constexpr u64 B_QS_SAFE = 0x0C00000000000000ull;
constexpr u64 B_QS_PATH = 0x0E00000000000000ull;

// CMove flags (chess.h:272-293)
enum : int {
    MF_QUIET = 0, MF_DOUBLE = 1, MF_KCASTLE = 2, MF_QCASTLE = 3, MF_CAPTURE = 4, MF_EP = 5,
    MF_PROMO_N = 8, MF_PROMO_B = 9, MF_PROMO_R = 10, MF_PROMO_Q = 11
};

__host__ __device__ __forceinline__ u16 cmove(int from, int to, int fl)
{
    return (u16)(((fl & 0xF) << 12) | ((to & 0x3F) << 6) | (from & 0x3F));
}

__device__ __forceinline__ int lsb(u64 x) { return __ffsll((long long)x) - 1; }
// the square of a one-bit set (count of leading zeros; 63 for an empty set)
__device__ __forceinline__ int sq_of(u64 one) { return (63 - __clzll((long long)one)) & 63; }
__device__ __forceinline__ int popc(u64 x) { return __popcll(x); }
__device__ __forceinline__ u64 lowbit(u64 x) { return x & (0ull - x); }
// more than one bit set: two 32-bit popcounts (off the ALU pipe) instead of
// the 64-bit x & (x - 1); 0.2-0.3% less leaf time, measured
__device__ __forceinline__ bool several(u64 x) { return __popc((u32)x) + __popc((u32)(x >> 32)) > 1; }

// ---- packed state ----
__device__ __forceinline__ int st_side(const Pos& b) { return (int)(b.p >> 63); }
__device__ __forceinline__ int st_wc(const Pos& b) { return (int)(b.p & 3); }
__device__ __forceinline__ int st_bc(const Pos& b) { return (int)((b.p >> 2) & 3); }
__device__ __forceinline__ int st_ep(const Pos& b) { return (int)((b.p >> 4) & 15); }
__device__ __forceinline__ void set_wc(Pos& b, int v) { b.p = (b.p & ~3ull) | (u64)(v & 3); }
__device__ __forceinline__ void set_bc(Pos& b, int v) { b.p = (b.p & ~12ull) | ((u64)(v & 3) << 2); }
__device__ __forceinline__ void set_ep(Pos& b, int v) { b.p = (b.p & ~0xF0ull) | ((u64)(v & 15) << 4); }
__device__ __forceinline__ void set_side(Pos& b, int v) { b.p = (b.p & ~(1ull << 63)) | ((u64)(v & 1) << 63); }
__device__ __forceinline__ void set_hm(Pos& b, int v) { b.p = (b.p & ~(0x7Full << 56)) | ((u64)(v & 0x7F) << 56); }

// ---- left shifts on the FMA pipe ----
// The move count is bound by integer-ALU issue (ALU pipe ~88-91% busy, FMA
// pipe ~10-14%).  The propagator chains' 64-bit left shifts are written as 32-bit
// multiplies by 2^K read from __constant__ memory, which the compiler cannot
// turn back into shifts: the low word one multiply, the high word one
// multiply-add of the bits carried over from the low word (one ALU shift).
// Two ALU shifts become one ALU shift and two FMA-pipe multiplies; measured
// 0.3% less leaf time on the batched workload, 0.9% less for the persistent
// launch.  (The same shifts as 64-bit wide and high-word multiplies were
// slower: those take more FMA-pipe issue.)
static __constant__ u32 g_pow2[32] = {1u, 2u, 4u, 8u, 16u, 32u, 64u, 128u, 256u, 512u, 1024u, 2048u, 4096u, 8192u,
                                      16384u, 32768u, 65536u, 131072u, 262144u, 524288u, 1048576u, 2097152u,
                                      4194304u, 8388608u, 16777216u, 33554432u, 67108864u, 134217728u, 268435456u,
                                      536870912u, 1073741824u, 2147483648u};
__device__ __forceinline__ u32 fmul32(u32 a, u32 m)
{
    u32 d;
    asm("mul.lo.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(m));
    return d;
}
__device__ __forceinline__ u32 fmad32(u32 a, u32 m, u32 c)
{
    u32 d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(m), "r"(c));
    return d;
}
// x << K (0 < K < 64)
template <int K> __device__ __forceinline__ u64 shl(u64 x)
{
    static_assert(K > 0 && K < 64, "shift out of range");
    const u32 lo = (u32)x, hi = (u32)(x >> 32);
    if constexpr (K >= 32) {
        return (u64)fmul32(lo, g_pow2[K - 32]) << 32;
    } else {
        return ((u64)fmad32(hi, g_pow2[K], lo >> (32 - K)) << 32) | fmul32(lo, g_pow2[K]);
    }
}

// ---- one-square steps ----
__device__ __forceinline__ u64 up(u64 x) { return x << 8; }
__device__ __forceinline__ u64 down(u64 x) { return x >> 8; }
__device__ __forceinline__ u64 east1(u64 x) { return (x << 1) & NOT_A; }
__device__ __forceinline__ u64 west1(u64 x) { return (x >> 1) & NOT_H; }
__device__ __forceinline__ u64 up_e(u64 x) { return (x << 9) & NOT_A; }
__device__ __forceinline__ u64 up_w(u64 x) { return (x << 7) & NOT_H; }
__device__ __forceinline__ u64 dn_e(u64 x) { return (x >> 7) & NOT_A; }
__device__ __forceinline__ u64 dn_w(u64 x) { return (x >> 9) & NOT_H; }

template <int S> __device__ __forceinline__ u64 push1(u64 x) { return S ? down(x) : up(x); }
template <int S> __device__ __forceinline__ u64 cap_w(u64 x) { return S ? dn_w(x) : up_w(x); }
template <int S> __device__ __forceinline__ u64 cap_e(u64 x) { return S ? dn_e(x) : up_e(x); }
// squares from which an enemy pawn (of side !S) attacks x, seen from side S
template <int S> __device__ __forceinline__ u64 pawn_attackers_of(u64 x) { return S ? (dn_e(x) | dn_w(x)) : (up_e(x) | up_w(x)); }
// squares attacked by pawns of side T
template <int T> __device__ __forceinline__ u64 pawn_attacks(u64 p) { return T ? (dn_e(p) | dn_w(p)) : (up_e(p) | up_w(p)); }
template <int S> __device__ __forceinline__ constexpr u64 double_rank() { return S ? RANK_6 : RANK_3; }

__device__ __forceinline__ u64 knight_set(u64 n)
{
    u64 a = ((n >> 1) & NOT_H) | ((n << 1) & NOT_A);
    u64 b = ((n >> 2) & 0x3F3F3F3F3F3F3F3Full) | ((n << 2) & 0xFCFCFCFCFCFCFCFCull);
    return (a << 16) | (a >> 16) | (b << 8) | (b >> 8);
}
__device__ __forceinline__ u64 king_set(u64 k)
{
    u64 a = east1(k) | west1(k);
    u64 row = k | a;
    return a | up(row) | down(row);
}

// ---- Kogge-Stone occluded fill in one direction ----
// SH: step (1, 7, 8 or 9); LEFT: toward higher squares; KEEP: wrap mask.
// Returns the squares attacked in that direction, first blocker included.
template <int SH, bool LEFT> __device__ __forceinline__ u64 shf(u64 x) { return LEFT ? (x << SH) : (x >> SH); }

template <int SH, bool LEFT> struct DirMask {
    static constexpr u64 keep = (SH == 8) ? ~0ull
                              : (SH == 1) ? (LEFT ? NOT_A : NOT_H)
                              : (SH == 9) ? (LEFT ? NOT_A : NOT_H)
                                          : (LEFT ? NOT_H : NOT_A);  // SH == 7
};

// propagator chain of one direction, shared by every generator filled along it
template <int SH, bool LEFT> struct Pro {
    u64 p1, p2, p4;
    __device__ __forceinline__ explicit Pro(u64 empty)
    {
        p1 = empty & DirMask<SH, LEFT>::keep;
        p2 = p1 & shf<SH, LEFT>(p1);
        p4 = p2 & shf<2 * SH, LEFT>(p2);
    }
    __device__ __forceinline__ u64 attacks(u64 g) const
    {
        g |= p1 & shf<SH, LEFT>(g);
        g |= p2 & shf<2 * SH, LEFT>(g);
        g |= p4 & shf<4 * SH, LEFT>(g);
        return shf<SH, LEFT>(g) & DirMask<SH, LEFT>::keep;
    }
};

template <int SH, bool LEFT> __device__ __forceinline__ u64 ray(u64 g, u64 empty)
{
    return Pro<SH, LEFT>(empty).attacks(g);
}

__device__ __forceinline__ u64 ks_bishop(u64 g, u64 empty)
{
    return ray<9, true>(g, empty) | ray<7, true>(g, empty) | ray<7, false>(g, empty) | ray<9, false>(g, empty);
}
// both vertical fills at once: with no wrap mask the down chain is the up
// chain shifted (p2 down = p2 up >> 8, p4 down = p4 up >> 24)
__device__ __forceinline__ void vertical_fills(u64 empty, u64 g, u64& up_att, u64& down_att)
{
    const u64 p2 = empty & (empty << 8), p4 = p2 & (p2 << 16);
    const u64 q2 = p2 >> 8, q4 = p4 >> 24;
    u64 a = g | (empty & (g << 8));
    a |= p2 & (a << 16);
    a |= p4 & (a << 32);
    up_att = a << 8;
    u64 c = g | (empty & (g >> 8));
    c |= q2 & (c >> 16);
    c |= q4 & (c >> 32);
    down_att = c >> 8;
}

// the same two chains kept for several generator sets
struct VPro {
    u64 e, p2, p4, q2, q4;
    __device__ __forceinline__ explicit VPro(u64 empty)
    {
        e = empty;
        p2 = empty & shl<8>(empty);
        p4 = p2 & shl<16>(p2);
        q2 = p2 >> 8;
        q4 = p4 >> 24;
    }
    __device__ __forceinline__ u64 up(u64 g) const
    {
        g |= e & shl<8>(g);
        g |= p2 & shl<16>(g);
        g |= p4 & (g << 32);
        return shl<8>(g);
    }
    __device__ __forceinline__ u64 down(u64 g) const
    {
        g |= e & (g >> 8);
        g |= q2 & (g >> 16);
        g |= q4 & (g >> 32);
        return g >> 8;
    }
};

// both directions of one diagonal line kind (SH = 9 or 7) from one chain.
// The chain holds the squares a ray passes THROUGH: empty and on neither edge
// file (a ray's inner squares never lie on the edge it moves away from, and
// it cannot pass the edge it moves toward), so it is the same for both
// directions and the backward chain is the forward one shifted back.
template <int SH> struct DPro {
    u64 p1, p2, p4, q2, q4;
    __device__ __forceinline__ explicit DPro(u64 pass)
    {
        p1 = pass;
        p2 = pass & shl<SH>(pass);
        p4 = p2 & shl<2 * SH>(p2);
        q2 = p2 >> SH;
        q4 = p4 >> (3 * SH);
    }
    __device__ __forceinline__ u64 up(u64 g) const
    {
        g |= p1 & shl<SH>(g);
        g |= p2 & shl<2 * SH>(g);
        g |= p4 & shl<4 * SH>(g);
        return shl<SH>(g) & DirMask<SH, true>::keep;
    }
    __device__ __forceinline__ u64 down(u64 g) const
    {
        g |= p1 & (g >> SH);
        g |= q2 & (g >> (2 * SH));
        g |= q4 & (g >> (4 * SH));
        return (g >> SH) & DirMask<SH, false>::keep;
    }
};

__device__ __forceinline__ u64 ks_rook(u64 g, u64 empty)
{
    return ray<8, true>(g, empty) | ray<8, false>(g, empty) | ray<1, true>(g, empty) | ray<1, false>(g, empty);
}

// the four lines through a square (used to split pinned pieces by pin line)
// both 32-bit halves of a file are the same: one 32-bit shift
__device__ __forceinline__ u64 file_of(int sq)
{
    const u32 h = 0x01010101u << (sq & 7);
    return ((u64)h << 32) | h;
}
__device__ __forceinline__ u64 rank_of(int sq) { return RANK_1 << (sq & 56); }
__device__ __forceinline__ u64 diag_of(int sq)
{
    int d = (sq >> 3) - (sq & 7);
    return d >= 0 ? (DIAG_A1H8 << (8 * d)) : (DIAG_A1H8 >> (-8 * d));
}
__device__ __forceinline__ u64 anti_of(int sq)
{
    int d = (sq >> 3) + (sq & 7) - 7;
    return d >= 0 ? (DIAG_A8H1 << (8 * d)) : (DIAG_A8H1 >> (-8 * d));
}

// squares strictly between lo and hi on the line `line`
__device__ __forceinline__ u64 between_on(u64 line, int a, int b)
{
    int lo = min(a, b), hi = max(a, b);
    return line & ((1ull << hi) - (2ull << lo));
}

}  // namespace pg
