// pg_movegen.cuh -- legal move generation for sm_103a, side-templated.
//
// Semantics follow the reference's MoveGeneratorBitboard (MGB.h below):
//   count_moves    <- countMoves<c>          MGB.h:3008-3295 (+2825-3002)
//   gen_moves      <- generateMoves<c>       MGB.h:2469-2823 (+2266-2463),
//                     host flavour (capture flag on non-pawn captures outside
//                     check, MGB.h:2525-2529); same order, same flags
//   make_move      <- makeMove<c,false>      MGB.h:3310-3570 with exact
//                     en-passant flagging (MGB.h:3528-3547)
//   gen_boards     <- generateBoards<c>      MGB.h:1940-2261 (+1741-1933,
//                     child boards as built by MGB.h:1302-1738)
// The legality rules are the reference's, including its behaviour on
// castling rights without a rook (no rook test) and on en passant while in
// check (only when the captured pawn is the checker).
//
// The formulation is our own and built for a 32-bit SIMT ALU: no per-thread
// colour branches (S is a template parameter and frontier ranges are
// side-uniform), own slider moves counted set-wise per direction with the
// Kogge-Stone policy (rays of different sliders along one direction are
// disjoint, so the popcounts add up exactly), and pins and checks found
// from the king's rays (two magic lookups) met by the enemy sliders' fills.
#pragma once
#include "pg_board.cuh"
#include "pg_tables.h"

namespace pg {

// ---------------------------------------------------------------------------
// slider attack policies
// ---------------------------------------------------------------------------

// Every translation unit that includes this header owns one copy of the
// tables (non-relocatable device code gives __device__ variables internal
// linkage) and uploads it through its own upload function at pg_init.
static __device__ __align__(16) MagicSq g_magic_rook[64];
static __device__ __align__(16) MagicSq g_magic_bishop[64];
static __device__ u64 g_magic_attacks[MAGIC_TABLE_ENTRIES];
static __device__ __align__(16) unsigned char g_magic_bytes[MAGIC_TABLE_ENTRIES];
static __device__ u64 g_magic_unique[UNIQUE_TOTAL];
static __device__ u64 g_knight[64];
// g_knight_t[s] = g_knight[s], g_knight_t[64] = 0: indexed by the number of
// squares below a set's lowest square (64 for an empty set), so a missing
// knight reads the zero entry and needs no mask or bit isolation (1.6% less
// leaf time than isolating the knight and masking g_knight's entry)
static __device__ u64 g_knight_t[65];
static __device__ u64 g_king[64];
static __device__ u64 g_diag[64];
static __device__ u64 g_pawn_checks[2][64];
// The count is bound by integer-ALU issue (the ALU pipe ~88-91% busy, the
// FMA pipe ~10-14%).  Its popcount sums are written as multiply-adds by a 1 the
// compiler cannot fold (a __constant__ word), so they issue on the FMA pipe
// instead of as ALU adds (measured 0.6% less leaf time on the batched
// workload).
static __constant__ u32 g_fma_one = 1;
__device__ __forceinline__ u32 fma_add(u32 a, u32 b)
{
    u32 d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(g_fma_one), "r"(b));
    return d;
}
// o - 2m per 32-bit half, as multiply-adds by -2 on the FMA pipe; equal to
// the 64-bit o - 2m when no borrow leaves bit 31 (bit 31 of o set).  The rank
// fills below subtract this way: 1.2% less leaf time on the batched workload
// than the 64-bit shift, mask and subtraction on the ALU pipe.
static __constant__ u32 g_fma_m2 = 0xFFFFFFFEu;
__device__ __forceinline__ u64 sub2_halves(u64 o, u64 m)
{
    u32 lo, hi;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(lo) : "r"((u32)m), "r"(g_fma_m2), "r"((u32)o));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(hi) : "r"((u32)(m >> 32)), "r"(g_fma_m2), "r"((u32)(o >> 32)));
    return ((u64)hi << 32) | lo;
}
// n + popcount(x), the additions on the FMA pipe
__device__ __forceinline__ u32 fma_popc(u32 n, u64 x) { return fma_add(__popc((u32)(x >> 32)), fma_add(__popc((u32)x), n)); }

// uploads this translation unit's copy of the tables
static inline cudaError_t upload_static_tables(const HostTables& t)
{
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(g_magic_rook, t.rook, sizeof(t.rook)))) return e;
    if ((e = cudaMemcpyToSymbol(g_magic_bishop, t.bishop, sizeof(t.bishop)))) return e;
    if ((e = cudaMemcpyToSymbol(g_magic_attacks, t.attacks.data(), t.attacks.size() * sizeof(u64)))) return e;
    if ((e = cudaMemcpyToSymbol(g_magic_bytes, t.bytes.data(), t.bytes.size()))) return e;
    if ((e = cudaMemcpyToSymbol(g_magic_unique, t.unique.data(), t.unique.size() * sizeof(u64)))) return e;
    if ((e = cudaMemcpyToSymbol(g_king, t.king, sizeof(t.king)))) return e;
    if ((e = cudaMemcpyToSymbol(g_diag, t.diag, sizeof(t.diag)))) return e;
    if ((e = cudaMemcpyToSymbol(g_pawn_checks, t.pawn_checks, sizeof(t.pawn_checks)))) return e;
    if ((e = cudaMemcpyToSymbol(g_knight, t.knight, sizeof(t.knight)))) return e;
    {
        u64 kt[65];
        for (int i = 0; i < 64; i++) kt[i] = t.knight[i];
        kt[64] = 0;
        if ((e = cudaMemcpyToSymbol(g_knight_t, kt, sizeof(kt)))) return e;
    }
    // uploads from pageable memory may still be in flight when these calls
    // return, and the kernels run on non-blocking streams: finish them here
    return cudaStreamSynchronize(0);
}

// Kogge-Stone: pure shift/and/or, no memory traffic.
struct SlKS {
    static constexpr int kId = 0;
    static constexpr bool kSetwise = true;
    __device__ __forceinline__ static u64 bishop(int sq, u64 occ) { return ks_bishop(1ull << sq, ~occ); }
    __device__ __forceinline__ static u64 rook(int sq, u64 occ) { return ks_rook(1ull << sq, ~occ); }
};

// fancy magics, 841 KB attack table read through the L1/L2 (ld.global.nc)
struct SlFancy {
    static constexpr int kId = 1;
    static constexpr bool kSetwise = false;
    __device__ __forceinline__ static u64 look(const MagicSq* t, int sq, u64 occ)
    {
        // one 32-byte entry as two 16-byte loads: (mask, magic), (offset, shift, ...)
        const uint4* e = reinterpret_cast<const uint4*>(t + sq);
        const uint4 a = __ldg(e), c = __ldg(e + 1);
        const u64 mask = ((u64)a.y << 32) | a.x, magic = ((u64)a.w << 32) | a.z;
        return __ldg(&g_magic_attacks[c.x + (u32)(((occ & mask) * magic) >> c.y)]);
    }
    __device__ __forceinline__ static u64 bishop(int sq, u64 occ) { return look(g_magic_bishop, sq, occ); }
    __device__ __forceinline__ static u64 rook(int sq, u64 occ) { return look(g_magic_rook, sq, occ); }
};

// byte-lookup fancy magics staged in shared memory (158 KB per CTA): the hash
// selects a byte, the byte selects one of the square's unique attack sets.
struct SmemTables {
    u64 unique[UNIQUE_TOTAL];
    MagicSq rook[64];
    MagicSq bishop[64];
    unsigned char bytes[MAGIC_TABLE_ENTRIES];
};
constexpr int SMEM_TABLE_BYTES = (int)sizeof(SmemTables);

struct SlByteSmem {
    static constexpr int kId = 2;
    static constexpr bool kSetwise = false;
    __device__ __forceinline__ static SmemTables* tab()
    {
        extern __shared__ __align__(16) unsigned char pg_dyn_smem[];
        return reinterpret_cast<SmemTables*>(pg_dyn_smem);
    }
    __device__ __forceinline__ static u64 look(const MagicSq& e, int sq, u64 occ)
    {
        const SmemTables* t = tab();
        u32 idx = e.offset + (u32)(((occ & e.mask) * e.magic) >> e.shift);
        return t->unique[e.uniq + t->bytes[idx]];
    }
    __device__ __forceinline__ static u64 bishop(int sq, u64 occ) { return look(tab()->bishop[sq], sq, occ); }
    __device__ __forceinline__ static u64 rook(int sq, u64 occ) { return look(tab()->rook[sq], sq, occ); }
    // every thread of the CTA calls this once before the first lookup
    __device__ static void stage()
    {
        SmemTables* t = tab();
        const int tid = threadIdx.x, nt = blockDim.x;
        const uint4* src_b = reinterpret_cast<const uint4*>(g_magic_bytes);
        uint4* dst_b = reinterpret_cast<uint4*>(t->bytes);
        for (int i = tid; i < MAGIC_TABLE_ENTRIES / 16; i += nt) dst_b[i] = __ldg(&src_b[i]);
        for (int i = tid; i < UNIQUE_TOTAL; i += nt) t->unique[i] = __ldg(&g_magic_unique[i]);
        for (int i = tid; i < 64; i += nt) {
            t->rook[i] = g_magic_rook[i];
            t->bishop[i] = g_magic_bishop[i];
        }
        __syncthreads();
    }
};

// hybrid: Kogge-Stone set-wise scans for the enemy's attacks, pins and checks
// (ALU), fancy-magic lookups for the own sliders' moves (multiply on the FMA
// pipe, table read on the load pipe), so the three pipes share the work
struct SlHybrid {
    static constexpr int kId = 3;
    static constexpr bool kSetwise = true;
    __device__ __forceinline__ static u64 bishop(int sq, u64 occ) { return SlFancy::bishop(sq, occ); }
    __device__ __forceinline__ static u64 rook(int sq, u64 occ) { return SlFancy::rook(sq, occ); }
};

template <class SL> __device__ __forceinline__ void stage_tables()
{
    if constexpr (SL::kId == 2) SlByteSmem::stage();
}
template <class SL> constexpr int table_smem_bytes() { return SL::kId == 2 ? SMEM_TABLE_BYTES : 0; }

template <class SL> __device__ __forceinline__ u64 bishops_of(u64 set, u64 occ)
{
    if constexpr (SL::kSetwise) {
        return ks_bishop(set, ~occ);
    } else {
        u64 a = 0;
        for (; set; set &= set - 1) a |= SL::bishop(lsb(set), occ);
        return a;
    }
}
template <class SL> __device__ __forceinline__ u64 rooks_of(u64 set, u64 occ)
{
    if constexpr (SL::kSetwise) {
        return ks_rook(set, ~occ);
    } else {
        u64 a = 0;
        for (; set; set &= set - 1) a |= SL::rook(lsb(set), occ);
        return a;
    }
}

// ---------------------------------------------------------------------------
// per-position facts
// ---------------------------------------------------------------------------

template <int S> struct Sides {
    u64 pawns, occ, mine, theirs, king, tbq, trq;
    int ksq;
    __device__ __forceinline__ explicit Sides(const Pos& b)
    {
        pawns = b.p & INNER;
        occ = b.k | pawns | b.n | b.bq | b.rq;
        const u64 black = occ & ~b.w;
        mine = S ? black : b.w;
        theirs = S ? b.w : black;
        king = b.k & mine;
        ksq = lsb(king) & 63;
        tbq = b.bq & theirs;
        trq = b.rq & theirs;
    }
};

// findPinnedPieces (MGB.h:1213-1249): the single piece between the king and
// an aligned enemy slider.  Aligned sliders are taken from the king's four
// lines, and the squares between from the line and the index range.
__device__ __forceinline__ u64 find_pinned(int ksq, u64 tbq, u64 trq, u64 occ)
{
    const u64 kb = 1ull << ksq;
    const u64 lf = file_of(ksq), lr = rank_of(ksq), ld = diag_of(ksq), la = anti_of(ksq);
    u64 cand = (((lf | lr) & trq) | ((ld | la) & tbq)) & ~kb;
    u64 pinned = 0;
    while (cand) {
        const int a = lsb(cand);
        const u64 ab = 1ull << a;
        const u64 line = (lf & ab) ? lf : (lr & ab) ? lr : (ld & ab) ? ld : la;
        const u64 inb = between_on(line, a, ksq) & occ;
        if (!several(inb)) pinned |= inb;
        cand &= cand - 1;
    }
    return pinned;
}

// the line through the king that holds square bit sb (0 when none)
__device__ __forceinline__ u64 king_line(int ksq, u64 sb)
{
    const u64 lf = file_of(ksq), lr = rank_of(ksq), ld = diag_of(ksq), la = anti_of(ksq);
    return (lf & sb) ? lf : (lr & sb) ? lr : (ld & sb) ? ld : (la & sb) ? la : 0ull;
}

// findAttackedSquares (MGB.h:1254-1298) with the own king removed
template <int S, class SL> __device__ __forceinline__ u64 threat_full(const Pos& b, const Sides<S>& c)
{
    const u64 occ_nk = c.occ & ~c.king;
    u64 t = pawn_attacks<1 - S>(c.pawns & c.theirs);
    t |= knight_set(b.n & c.theirs);
    t |= king_set(b.k & c.theirs);
    t |= bishops_of<SL>(c.tbq, occ_nk);
    t |= rooks_of<SL>(c.trq, occ_nk);
    return t;
}

template <int S> __device__ __forceinline__ u64 ep_target(const Pos& b)
{
    const int ep = st_ep(b);
    return ep ? ((1ull << (ep - 1)) << (S ? 16 : 40)) : 0ull;
}

template <int S> __device__ __forceinline__ bool can_castle_k(const Pos& b, u64 occ, u64 threat)
{
    if (S == 0) return (st_wc(b) & 1) && !(W_KS_PATH & occ) && !(W_KS_PATH & threat);
    return (st_bc(b) & 1) && !(B_KS_PATH & occ) && !(B_KS_PATH & threat);
}
template <int S> __device__ __forceinline__ bool can_castle_q(const Pos& b, u64 occ, u64 threat)
{
    if (S == 0) return (st_wc(b) & 2) && !(W_QS_PATH & occ) && !(W_QS_SAFE & threat);
    return (st_bc(b) & 2) && !(B_QS_PATH & occ) && !(B_QS_SAFE & threat);
}

// en passant outside check (MGB.h:3058-3093): a pinned capturer must stay on
// its pin line; otherwise the rank of the two pawns must not open onto the king
template <int S> __device__ __forceinline__ bool ep_legal(const Sides<S>& c, u64 pinned, u64 pawn, u64 tgt, u64 victim)
{
    if (pawn & pinned) return (tgt & king_line(c.ksq, pawn)) != 0;
    const u64 pro = ~c.occ | victim | pawn;
    return ((ray<1, true>(c.trq, pro) | ray<1, false>(c.trq, pro)) & c.king) == 0;
}

// checkers of the king (MGB.h:2842-2860)
template <int S, class SL> __device__ __forceinline__ u64 checkers(const Pos& b, const Sides<S>& c)
{
    u64 a = pawn_attackers_of<S>(c.king) & (c.pawns & c.theirs);
    a |= knight_set(c.king) & (b.n & c.theirs);
    a |= SL::bishop(c.ksq, c.occ) & c.tbq;
    a |= SL::rook(c.ksq, c.occ) & c.trq;
    return a;
}

// ---------------------------------------------------------------------------
// countMoves
// ---------------------------------------------------------------------------

// Enemy slider attacks along one line kind (both directions of one step),
// filled through `empty`.
template <int SH> __device__ __forceinline__ u64 line_fill(u64 empty, u64 sliders)
{
    return Pro<SH, true>(empty).attacks(sliders) | Pro<SH, false>(empty).attacks(sliders);
}

// en passant for the branch-free count (rare: the file is set only when a
// capture is possible).  Outside check: MGB.h:3058-3093; in check only when
// the pushed pawn is the single checker (MGB.h:2903-2906, 2948-2953).
template <int S>
__device__ __noinline__ u32 count_ep_ks(const Pos& b, u64 pinned, u64 checkers)
{
    const Sides<S> c(b);
    const u64 tgt = ep_target<S>(b);
    const u64 victim = S ? up(tgt) : down(tgt);
    const u64 myp = c.pawns & c.mine;
    if (checkers) {
        if (victim != checkers) return 0;
        const u64 fp = myp & ~pinned;
        return popc(cap_w<S>(fp) & tgt) + popc(cap_e<S>(fp) & tgt);
    }
    u32 n = 0;
    for (u64 s = (east1(victim) | west1(victim)) & myp; s; s &= s - 1)
        n += ep_legal<S>(c, pinned, lowbit(s), tgt, victim) ? 1 : 0;
    return n;
}

// What the count and the in-kernel generator need to know about a position,
// computed without a branch: pins per line, checkers, the target mask and
// the squares the enemy attacks with the side to move's king taken off the
// board (findPinnedPieces / findAttackedSquares, MGB.h:1213-1298, in mask
// form).
template <int S> struct KsFacts {
    u64 pawns, occ, mine, theirs, empty;
    int ksq;
    u64 pf, pr, pd, pa;  // own pieces pinned along the king's file / rank / diagonal / anti-diagonal
    u64 pinned, checkers;
    u64 safe;     // the check ray and the checkers (nothing out of check)
    u64 threat;   // enemy attacks with the king transparent
    u64 chk_all;  // all ones in check
    u64 tgt;      // where non-king pieces may move: ~own, the check ray, or nothing
};

template <int S> __device__ __forceinline__ KsFacts<S> ks_facts(const Pos& b)
{
    KsFacts<S> f;
    const u64 pawns = b.p & INNER;
    const u64 occ = b.k | pawns | b.n | b.bq | b.rq;
    const u64 black = occ & ~b.w;
    const u64 mine = S ? black : b.w, theirs = S ? b.w : black;
    const u64 king = b.k & mine;
    const u64 empty = ~occ;
    const u64 trq = b.rq & theirs, tbq = b.bq & theirs;
    const u64 tp = pawns & theirs, tn = b.n & theirs;

    // enemy slider fills per line kind, with the king taken off the board so
    // that the squares behind it on a checking line are attacked
    const u64 et = empty | king;
    u64 a_up, a_dn;
    vertical_fills(et, trq, a_up, a_dn);
    const u64 a_v = a_up | a_dn, a_h = line_fill<1>(et, trq);
    const u64 a_d = line_fill<9>(et, tbq), a_a = line_fill<7>(et, tbq);

    // the king's rays (first blockers included): one rook and one bishop
    // lookup, split into the four lines
    const int ksq = sq_of(king);
    const u64 kr = SlFancy::rook(ksq, occ), kb = SlFancy::bishop(ksq, occ);
    const u64 kf = kr & file_of(ksq), kd = kb & __ldg(&g_diag[ksq]);
    const u64 kh = kr ^ kf, ka = kb ^ kd;

    // A first blocker of the king on a line is pinned when an enemy slider
    // attacks it along that line: nothing lies between the king and it, so
    // the attack comes from beyond it.  With the king transparent, a slider
    // checking along a line also reaches the king's first blocker on the far
    // side; that piece can neither capture the checker nor block (every route
    // onto the checking line crosses the king), and pinned pieces do not move
    // in check, so the moves are the same.
    f.pf = kf & a_v & mine;
    f.pr = kh & a_h & mine;
    f.pd = kd & a_d & mine;
    f.pa = ka & a_a & mine;
    f.pinned = f.pf | f.pr | f.pd | f.pa;
    const u64 cr = kr & trq, cb = kb & tbq;
    const u64 nchk = __ldg(&g_knight[ksq]) & tn;
    const u64 pchk = __ldg(&g_pawn_checks[S][ksq]) & tp;
    const u64 csl = cr | cb;
    f.checkers = csl | nchk | pchk;
    // single slider check: the squares between the king and the checker are
    // where the king's rays meet the checker's rays of the same kind (the
    // other lines of the two pieces are parallel); looked up by every lane
    // when any lane of the warp has a slider checker (no divergence), and
    // dropped where no slider checks
    const int csq = lsb(csl) & 63;
    u64 cray = 0;
    if (__any_sync(__activemask(), csl != 0))
        cray = SlFancy::look(cr ? g_magic_rook : g_magic_bishop, csq, occ) & (cr ? kr : kb);
    f.safe = (csl ? cray : 0ull) | f.checkers;
    f.threat = a_v | a_h | a_d | a_a | pawn_attacks<1 - S>(tp) | knight_set(tn) | __ldg(&g_king[sq_of(b.k & theirs)]);
    const bool in_check = f.checkers != 0;
    f.chk_all = in_check ? ~0ull : 0ull;
    f.tgt = several(f.checkers) ? 0ull : (in_check ? f.safe : ~mine);
    f.pawns = pawns;
    f.occ = occ;
    f.mine = mine;
    f.theirs = theirs;
    f.empty = empty;
    f.ksq = ksq;
    return f;
}

// countMoves / countMovesOutOfCheck (MGB.h:3008-3295, 2825-3002) as one
// instruction stream for the Kogge-Stone policy.  Check handling is a target
// mask: ~own outside check, the check ray (between squares + checker) in
// single check, nothing in double check; pinned pieces move along their pin
// line outside check and not at all in check.  The counts are the
// reference's in every case (proved per term in the comments of the
// reference-shaped paths above and checked bit-exact by the tests).
template <int S, bool OWN_BY_LOOKUP = false>
__device__ __forceinline__ u32 count_from_facts(const Pos& b, const KsFacts<S>& f)
{
    const u64 pawns = f.pawns, occ = f.occ, mine = f.mine, theirs = f.theirs, empty = f.empty;
    const u64 pf = f.pf, pr = f.pr, pd = f.pd, pa = f.pa, pinned = f.pinned, checkers = f.checkers;
    const u64 safe = f.safe, threat = f.threat, chk_all = f.chk_all, tgt = f.tgt;
    const int ksq = f.ksq;
    const bool in_check = checkers != 0;

    u32 n = popc(__ldg(&g_king[ksq]) & ~(threat | mine));

    const u64 my_rq = b.rq & mine, my_bq = b.bq & mine;
    const u64 pin_chk = pinned & chk_all;
    if constexpr (OWN_BY_LOOKUP) {
        // pass 2 by table lookup, one per own slider; a pinned piece keeps the
        // moves along its pin line (none if the line is not its kind)
        for (u64 s = my_rq & ~pin_chk; s; s &= s - 1) {
            const int sq = lsb(s);
            const u64 bit = 1ull << sq;
            u64 m = SlFancy::rook(sq, b.k | pawns | b.n | b.bq | b.rq) & tgt;
            if (pinned & bit) m &= (pf & bit) ? file_of(ksq) : (pr & bit) ? rank_of(ksq) : 0ull;
            n += popc(m);
        }
        for (u64 s = my_bq & ~pin_chk; s; s &= s - 1) {
            const int sq = lsb(s);
            const u64 bit = 1ull << sq;
            u64 m = SlFancy::bishop(sq, b.k | pawns | b.n | b.bq | b.rq) & tgt;
            if (pinned & bit) m &= (pd & bit) ? diag_of(ksq) : (pa & bit) ? anti_of(ksq) : 0ull;
            n += popc(m);
        }
    } else {
        // pass 2: own slider moves, through the real empty squares (pass 1's
        // chains treat the king as empty).  The chains are built from an
        // opaque copy of `empty`, so the compiler builds them here rather than
        // early, where they would be live across pass 1.
        u64 empty2 = empty;
        asm volatile("" : "+l"(empty2));
        {
            const u64 ns = my_rq & ~((pinned ^ pf) | pin_chk);
            u64 up_att, down_att;
            vertical_fills(empty2, ns, up_att, down_att);
            n += popc(up_att & tgt) + popc(down_att & tgt);
        }
        {
            const u64 ew = my_rq & ~((pinned ^ pr) | pin_chk);
            n += popc(Pro<1, true>(empty2).attacks(ew) & tgt) + popc(Pro<1, false>(empty2).attacks(ew) & tgt);
        }
        {
            const u64 dg = my_bq & ~((pinned ^ pd) | pin_chk);
            n += popc(Pro<9, true>(empty2).attacks(dg) & tgt) + popc(Pro<9, false>(empty2).attacks(dg) & tgt);
        }
        {
            const u64 ad = my_bq & ~((pinned ^ pa) | pin_chk);
            n += popc(Pro<7, true>(empty2).attacks(ad) & tgt) + popc(Pro<7, false>(empty2).attacks(ad) & tgt);
        }
    }

    for (u64 s = b.n & mine & ~pinned; s; s &= s - 1) n += popc(__ldg(&g_knight[lsb(s)]) & tgt);

    // pawns: pushes by free pawns and file-pinned pawns, captures by free
    // pawns and pawns pinned on that capture's diagonal; pinned pawns only
    // outside check.  In check a double push counts only when the single
    // push does not already answer the check.
    const u64 myp = pawns & mine;
    const u64 fp = myp & ~pinned;
    const u64 pin_ok = ~chk_all;
    const u64 d1 = push1<S>(fp | (myp & pf & pin_ok)) & empty;
    const u64 s1 = d1 & tgt;
    n += popc(s1) + 3 * popc(s1 & BACK_RANKS);
    n += popc(push1<S>(d1 & double_rank<S>() & ~safe) & empty & tgt);
    const u64 cw = cap_w<S>(fp | (myp & (S ? pd : pa) & pin_ok)) & theirs & tgt;
    const u64 ce = cap_e<S>(fp | (myp & (S ? pa : pd) & pin_ok)) & theirs & tgt;
    n += popc(cw) + popc(ce) + 3 * (popc(cw & BACK_RANKS) + popc(ce & BACK_RANKS));

    if (!in_check) n += can_castle_k<S>(b, occ, threat) + can_castle_q<S>(b, occ, threat);
    if (b.p & 0xF0ull) n += count_ep_ks<S>(b, pinned, checkers);
    return n;
}

template <int S, bool OWN_BY_LOOKUP = false>
__device__ __forceinline__ u32 count_moves_ks(const Pos& b)
{
    return count_from_facts<S, OWN_BY_LOOKUP>(b, ks_facts<S>(b));
}

// Rank attacks by subtraction: with file H marked occupied (so that no borrow
// leaves a rank), `o - 2g` borrows from each slider's next square up to its
// first blocker, and `o ^ (o - 2g)` is every slider's eastward ray, blocker
// included.  Rays of different sliders are disjoint, so the borrows never
// meet.  Sliders on file H have no eastward ray and are dropped before the
// doubling; as no borrow leaves a rank, none crosses from the low word to
// the high word, and the subtraction runs per 32-bit half (sub2_halves).
// Westward rays are the same on the bit-reversed board (file A <-> H).
struct RankPro {
    u64 oe, ow;
    __device__ __forceinline__ explicit RankPro(u64 occ)
    {
        oe = occ | FILE_H;
        ow = __brevll(occ | FILE_A);
    }
    __device__ __forceinline__ u64 east(u64 g) const { return oe ^ sub2_halves(oe, g & NOT_H); }
    __device__ __forceinline__ u64 west(u64 g) const
    {
        return __brevll(ow ^ sub2_halves(ow, __brevll(g) & NOT_H));
    }
};

// The same count with one propagator chain per direction, built from the
// real empty squares and shared by the enemy's sliders (attacks, pins) and
// the side to move's sliders (moves).  Three differences from ks_facts +
// count_from_facts make that possible:
//  * the king is opaque to the enemy fills, so the square behind the king on
//    a slider-checking line is added to the enemy attacks by hand (the
//    king's neighbour on the same king ray, on the far side from the checker);
//    outside check no enemy fill reaches the king and nothing differs;
//  * own sliders are filled as if none were pinned: rays of different
//    sliders along one direction are disjoint, so the filled popcounts are the
//    sum of every slider's own moves, and a pinned slider's moves off its pin
//    line (all of them in check) are taken back with one lookup per pinned
//    slider (rare);
//  * the checkers and the target mask come first (from the king's rays), so
//    each direction's own fill is counted as soon as it is made.
template <int S>
__device__ __forceinline__ u32 count_moves_ks1(const Pos& b)
{
    const u64 pawns = b.p & INNER;
    const u64 occ = b.k | pawns | b.n | b.bq | b.rq;
    const u64 black = occ & ~b.w;
    const u64 mine = S ? black : b.w, theirs = S ? b.w : black;
    const u64 king = b.k & mine;
    const u64 empty = ~occ;
    const u64 trq = b.rq & theirs, tbq = b.bq & theirs;
    const u64 my_rq = b.rq & mine, my_bq = b.bq & mine;
    const u64 tp = pawns & theirs, tn = b.n & theirs;

    // the king's rays, split per line, and the checkers
    const int ksq = sq_of(king);
    const u64 kr = SlFancy::rook(ksq, occ), kb = SlFancy::bishop(ksq, occ);
    const u64 kf = kr & file_of(ksq), kd = kb & __ldg(&g_diag[ksq]);
    const u64 kh = kr ^ kf, ka = kb ^ kd;
    const u64 cr = kr & trq, cb = kb & tbq;
    const u64 csl = cr | cb;
    const u64 checkers = csl | (__ldg(&g_knight[ksq]) & tn) | (__ldg(&g_pawn_checks[S][ksq]) & tp);
    u64 cray = 0, behind = 0;
    if (__any_sync(__activemask(), csl != 0)) {
        const int csq = lsb(csl) & 63;
        cray = SlFancy::look(cr ? g_magic_rook : g_magic_bishop, csq, occ) & (cr ? kr : kb);
        for (u64 s = csl; s; s &= s - 1) {
            const u64 c = s & (0ull - s);
            const u64 kray = (c & kf) ? kf : (c & kh) ? kh : (c & kd) ? kd : ka;
            behind |= kray & (c > king ? king - 1ull : ~(king | (king - 1ull)));
        }
    }
    const bool in_check = checkers != 0;
    const u64 chk_all = in_check ? ~0ull : 0ull;
    const u64 safe = (csl ? cray : 0ull) | checkers;
    const u64 tgt = several(checkers) ? 0ull : (in_check ? safe : ~mine);

    u32 n = 0;
    u64 threat, pf, pr, pd, pa;
    {
        const VPro v(empty);
        const u64 a_v = v.up(trq) | v.down(trq);
        pf = kf & a_v & mine;
        threat = a_v;
        n = fma_popc(fma_popc(n, v.up(my_rq) & tgt), v.down(my_rq) & tgt);
    }
    {
        const RankPro h(occ);
        const u64 a_h = h.east(trq) | h.west(trq);
        pr = kh & a_h & mine;
        threat |= a_h;
        n = fma_popc(fma_popc(n, h.east(my_rq) & tgt), h.west(my_rq) & tgt);
    }
    const u64 pass = empty & NOT_A & NOT_H;
    {
        const DPro<9> d(pass);
        const u64 a_d = d.up(tbq) | d.down(tbq);
        pd = kd & a_d & mine;
        threat |= a_d;
        n = fma_popc(fma_popc(n, d.up(my_bq) & tgt), d.down(my_bq) & tgt);
    }
    {
        const DPro<7> d(pass);
        const u64 a_a = d.up(tbq) | d.down(tbq);
        pa = ka & a_a & mine;
        threat |= a_a;
        n = fma_popc(fma_popc(n, d.up(my_bq) & tgt), d.down(my_bq) & tgt);
    }
    const u64 pinned = pf | pr | pd | pa;
    threat |= pawn_attacks<1 - S>(tp) | knight_set(tn) | __ldg(&g_king[sq_of(b.k & theirs)]);
    n = fma_popc(n, __ldg(&g_king[ksq]) & ~(threat | behind | mine));

    // pinned sliders: take back the moves off the pin line (all in check)
    for (u64 s = pinned & (my_rq | my_bq); s; s &= s - 1) {
        const int sq = lsb(s);
        const u64 bit = 1ull << sq;
        u64 att = (my_rq & bit) ? SlFancy::rook(sq, occ) : 0ull;
        if (my_bq & bit) att |= SlFancy::bishop(sq, occ);
        const u64 line = (pf & bit) ? file_of(ksq) : (pr & bit) ? rank_of(ksq)
                       : (pd & bit) ? __ldg(&g_diag[ksq]) : anti_of(ksq);
        n -= popc(att & tgt & ~(line & ~chk_all));
    }

    {
        // the first two knights without a loop (fewer instructions and no
        // divergence on the usual one or two): each one's square is the
        // popcount of the squares below it, 64 (the zero entry) when there
        // is none; a third (promotions) loops
        const u64 kn = b.n & mine & ~pinned;
        const u64 km = kn - 1, rest = kn & km, rm = rest - 1;
        const u64 t1 = ~kn & km, t2 = ~rest & rm;  // below the first / second knight (all ones if none)
        n = fma_popc(n, __ldg(&g_knight_t[__popc((u32)t1) + __popc((u32)(t1 >> 32))]) & tgt);
        n = fma_popc(n, __ldg(&g_knight_t[__popc((u32)t2) + __popc((u32)(t2 >> 32))]) & tgt);
        for (u64 s = rest & rm; s; s &= s - 1) n = fma_popc(n, __ldg(&g_knight[lsb(s)]) & tgt);
    }

    // pawns, castling and en passant as in count_from_facts
    const u64 myp = pawns & mine;
    const u64 fp = myp & ~pinned;
    const u64 pin_ok = ~chk_all;
    const u64 d1 = push1<S>(fp | (myp & pf & pin_ok)) & empty;
    const u64 s1 = d1 & tgt;
    // a promotion lands on the far back rank only: one 32-bit half
    n = fma_popc(n, s1) + 3 * __popc(S ? (u32)s1 & 0xFFu : (u32)(s1 >> 32) & 0xFF000000u);
    n = fma_popc(n, push1<S>(d1 & double_rank<S>() & ~safe) & empty & tgt);
    const u64 cw = cap_w<S>(fp | (myp & (S ? pd : pa) & pin_ok)) & theirs & tgt;
    const u64 ce = cap_e<S>(fp | (myp & (S ? pa : pd) & pin_ok)) & theirs & tgt;
    n = fma_popc(fma_popc(n, cw), ce) +
        3 * (S ? __popc((u32)cw & 0xFFu) + __popc((u32)ce & 0xFFu)
               : __popc((u32)(cw >> 32) & 0xFF000000u) + __popc((u32)(ce >> 32) & 0xFF000000u));

    // castling only when the side to move still holds a right (random
    // playouts lose them early: 1% less leaf time on the batched workload)
    if (!in_check && (b.p & (S ? 0xCull : 0x3ull)))
        n += can_castle_k<S>(b, occ, threat) + can_castle_q<S>(b, occ, threat);
    if (b.p & 0xF0ull) n += count_ep_ks<S>(b, pinned, checkers);
    return n;
}

// countMoves / countMovesOutOfCheck (MGB.h:3008-3295, 2825-3002) for the
// table policies, in the same mask form as count_moves_ks: one lookup per
// slider for the enemy attacks and for the own moves (the 64-bit multiply
// runs on the FMA pipe, the table read on the load pipe), two lookups from
// the king square for checks, and two x-ray lookups through the king's own
// first blockers for pins.  A pinner's rays meet the king's rays only on the
// pin line (the pinner's other line is parallel to the king's other line of
// the same kind), so `own first blockers & pinner attacks` is exactly the
// pinned piece.
template <int S, class SL>
__device__ __forceinline__ u32 count_moves_mg(const Pos& b)
{
    const u64 pawns = b.p & INNER;
    const u64 occ = b.k | pawns | b.n | b.bq | b.rq;
    const u64 black = occ & ~b.w;
    const u64 mine = S ? black : b.w, theirs = S ? b.w : black;
    const u64 king = b.k & mine;
    const int ksq = lsb(king) & 63;
    const u64 empty = ~occ;
    const u64 trq = b.rq & theirs, tbq = b.bq & theirs;
    const u64 tp = pawns & theirs, tn = b.n & theirs;

    u64 threat = pawn_attacks<1 - S>(tp) | knight_set(tn) | __ldg(&g_king[sq_of(b.k & theirs)]);
    for (u64 s = trq; s; s &= s - 1) threat |= SL::rook(lsb(s), occ);
    for (u64 s = tbq; s; s &= s - 1) threat |= SL::bishop(lsb(s), occ);

    const u64 ra = SL::rook(ksq, occ), ba = SL::bishop(ksq, occ);
    const u64 nchk = __ldg(&g_knight[ksq]) & tn;
    const u64 pchk = pawn_attackers_of<S>(king) & tp;
    const u64 schk = (ra & trq) | (ba & tbq);
    const u64 checkers = schk | nchk | pchk;
    u64 safe = nchk | pchk;
    u64 behind = 0;  // squares a checking slider attacks through the king
    for (u64 s = schk; s; s &= s - 1) {
        const int c = lsb(s);
        const u64 cb = 1ull << c;
        const bool orth = (ra & cb) != 0;
        safe |= ((orth ? ra : ba) & (orth ? SL::rook(c, occ) : SL::bishop(c, occ))) | cb;
        behind |= orth ? SL::rook(c, occ ^ king) : SL::bishop(c, occ ^ king);
    }
    const u64 rb = ra & mine, bb = ba & mine;
    const u64 pin_r = SL::rook(ksq, occ ^ rb) & ~ra & trq;
    const u64 pin_b = SL::bishop(ksq, occ ^ bb) & ~ba & tbq;
    u64 pinned = 0;
    for (u64 s = pin_r; s; s &= s - 1) pinned |= rb & SL::rook(lsb(s), occ);
    for (u64 s = pin_b; s; s &= s - 1) pinned |= bb & SL::bishop(lsb(s), occ);

    const bool in_check = checkers != 0;
    const u64 chk_all = in_check ? ~0ull : 0ull;
    const u64 tgt = several(checkers) ? 0ull : (in_check ? safe : ~mine);
    u32 n = popc(__ldg(&g_king[ksq]) & ~(threat | behind | mine));

    const u64 lf = file_of(ksq), lr = rank_of(ksq), ld = diag_of(ksq), la = anti_of(ksq);
    const u64 stay = pinned & chk_all;  // in check a pinned piece never moves
    for (u64 s = b.rq & mine & ~stay; s; s &= s - 1) {
        const int sq = lsb(s);
        const u64 bit = 1ull << sq;
        const u64 line = (pinned & bit) ? ((lf & bit) ? lf : (lr & bit) ? lr : (ld & bit) ? ld : la) : ~0ull;
        n += popc(SL::rook(sq, occ) & tgt & line);
    }
    for (u64 s = b.bq & mine & ~stay; s; s &= s - 1) {
        const int sq = lsb(s);
        const u64 bit = 1ull << sq;
        const u64 line = (pinned & bit) ? ((lf & bit) ? lf : (lr & bit) ? lr : (ld & bit) ? ld : la) : ~0ull;
        n += popc(SL::bishop(sq, occ) & tgt & line);
    }
    for (u64 s = b.n & mine & ~pinned; s; s &= s - 1) n += popc(__ldg(&g_knight[lsb(s)]) & tgt);

    const u64 myp = pawns & mine;
    const u64 fp = myp & ~pinned;
    const u64 pin_ok = ~chk_all;
    const u64 d1 = push1<S>(fp | (myp & pinned & lf & pin_ok)) & empty;
    const u64 s1 = d1 & tgt;
    n += popc(s1) + 3 * popc(s1 & BACK_RANKS);
    n += popc(push1<S>(d1 & double_rank<S>() & ~safe) & empty & tgt);
    const u64 cw = cap_w<S>(fp | (myp & pinned & (S ? ld : la) & pin_ok)) & theirs & tgt;
    const u64 ce = cap_e<S>(fp | (myp & pinned & (S ? la : ld) & pin_ok)) & theirs & tgt;
    n += popc(cw) + popc(ce) + 3 * (popc(cw & BACK_RANKS) + popc(ce & BACK_RANKS));

    if (!in_check) n += can_castle_k<S>(b, occ, threat) + can_castle_q<S>(b, occ, threat);
    if (b.p & 0xF0ull) n += count_ep_ks<S>(b, pinned, checkers);
    return n;
}

// countMoves (MGB.h:3008-3295)
template <int S, class SL>
__device__ __forceinline__ u32 count_moves(const Pos& b)
{
    if constexpr (SL::kId == 0) return count_moves_ks1<S>(b);
    else if constexpr (SL::kId == 3) return count_moves_ks<S, true>(b);
    else return count_moves_mg<S, SL>(b);
}

// ---------------------------------------------------------------------------
// generateMoves (reference order, host flags)
// ---------------------------------------------------------------------------

// addCompactPawnMoves (MGB.h:1717-1738): promotions N, B, Q, R
template <class E> __device__ __forceinline__ void emit_pawn(E& emit, int from, u64 dst, int fl)
{
    const int to = lsb(dst);
    if (dst & BACK_RANKS) {
        emit(cmove(from, to, fl | MF_PROMO_N));
        emit(cmove(from, to, fl | MF_PROMO_B));
        emit(cmove(from, to, fl | MF_PROMO_Q));
        emit(cmove(from, to, fl | MF_PROMO_R));
    } else {
        emit(cmove(from, to, fl));
    }
}

// The legal moves counted by count_moves_ks, emitted in an order of our own
// for the kernels that only need the set of children (the leaf and the level
// expansion): king, knights, bishop/queen, rook/queen, pawn pushes, double
// pushes, captures, castles, en passant.  Same analysis as the count, so the
// number emitted equals the count for every position.  The flags are the
// reference's where making the move reads them (double push, castles, en
// passant, promotions); captures carry no flag (makeMove clears the target
// square whatever the flag).
// Non-pawn moves also pass the moving piece (PC_*) to the emitter.
enum : u32 { PC_PAWN = 0, PC_KNIGHT = 1, PC_BISHOP = 2, PC_ROOK = 3, PC_QUEEN = 4, PC_KING = 5 };
// with a double push: an enemy pawn stands beside the pushed pawn, so the
// child's en-passant file is set (exact flagging, decided by the parent)
constexpr u32 PC_EP_FLAG = 8;
// calls f(square) for every square of m in ascending order (the order of a
// 64-bit lowest-bit loop), as two loops over the 32-bit halves: 32-bit
// find-first-set and clear-lowest instead of their 64-bit forms, 1.2-1.4%
// less leaf time (the leaf emits one queue entry per child)
template <class F> __device__ __forceinline__ void each_square(u64 m, F&& f)
{
    for (u32 x = (u32)m; x; x &= x - 1) f(__ffs(x) - 1);
    for (u32 x = (u32)(m >> 32); x; x &= x - 1) f(__ffs(x) + 31);
}
// a pawn move for the leaf, by target square: on rank 1 or 8 the promotions
// N, B, Q, R (the reference's flags) with the promoted piece as the landing
// piece
template <class E> __device__ __forceinline__ void emit_pawn_sq(E& emit, int from, int to, int fl)
{
    if ((u32)(to - 8) >= 48u) {
        emit(cmove(from, to, fl | MF_PROMO_N), PC_KNIGHT);
        emit(cmove(from, to, fl | MF_PROMO_B), PC_BISHOP);
        emit(cmove(from, to, fl | MF_PROMO_Q), PC_QUEEN);
        emit(cmove(from, to, fl | MF_PROMO_R), PC_ROOK);
    } else {
        emit(cmove(from, to, fl), PC_PAWN);
    }
}

template <int S, class E> __device__ __forceinline__ void gen_from_facts(const Pos& b, const KsFacts<S>& f, E& emit)
{
    const u64 tgt = f.tgt;
    const int ksq = f.ksq;
    each_square(__ldg(&g_king[ksq]) & ~(f.threat | f.mine), [&](int to) { emit(cmove(ksq, to, 0), PC_KING); });
    const u64 pin_chk = f.pinned & f.chk_all;
    for (u64 s = b.n & f.mine & ~f.pinned; s; s &= s - 1) {
        const int sq = lsb(s);
        each_square(__ldg(&g_knight[sq]) & tgt, [&](int to) { emit(cmove(sq, to, 0), PC_KNIGHT); });
    }
    // a pinned slider keeps the moves along its pin line (none if the line is
    // not its kind); in check pinned pieces do not move
    for (u64 s = b.bq & f.mine & ~pin_chk; s; s &= s - 1) {
        const int sq = lsb(s);
        const u64 bit = lowbit(s);
        u64 m = SlFancy::bishop(sq, f.occ) & tgt;
        if (f.pinned & bit) m &= (f.pd & bit) ? diag_of(ksq) : (f.pa & bit) ? anti_of(ksq) : 0ull;
        const u32 pc = (b.rq & bit) ? PC_QUEEN : PC_BISHOP;
        each_square(m, [&](int to) { emit(cmove(sq, to, 0), pc); });
    }
    for (u64 s = b.rq & f.mine & ~pin_chk; s; s &= s - 1) {
        const int sq = lsb(s);
        const u64 bit = lowbit(s);
        u64 m = SlFancy::rook(sq, f.occ) & tgt;
        if (f.pinned & bit) m &= (f.pf & bit) ? file_of(ksq) : (f.pr & bit) ? rank_of(ksq) : 0ull;
        const u32 pc = (b.bq & bit) ? PC_QUEEN : PC_ROOK;
        each_square(m, [&](int to) { emit(cmove(sq, to, 0), pc); });
    }
    // pawns, set-wise as in the count; from = to - step
    constexpr int PUSH = S ? -8 : 8, CW = S ? -9 : 7, CE = S ? -7 : 9;
    const u64 myp = f.pawns & f.mine;
    const u64 fp = myp & ~f.pinned;
    const u64 pin_ok = ~f.chk_all;
    const u64 d1 = push1<S>(fp | (myp & f.pf & pin_ok)) & f.empty;
    each_square(d1 & tgt, [&](int to) { emit_pawn_sq(emit, to - PUSH, to, 0); });
    const u64 their_pawns = f.pawns & f.theirs;
    for (u64 m = push1<S>(d1 & double_rank<S>() & ~f.safe) & f.empty & tgt; m; m &= m - 1) {
        const u64 t = lowbit(m);
        emit(cmove(lsb(m) - 2 * PUSH, lsb(m), MF_DOUBLE),
             PC_PAWN | (((east1(t) | west1(t)) & their_pawns) ? PC_EP_FLAG : 0u));
    }
    each_square(cap_w<S>(fp | (myp & (S ? f.pd : f.pa) & pin_ok)) & f.theirs & tgt,
                [&](int to) { emit_pawn_sq(emit, to - CW, to, 0); });
    each_square(cap_e<S>(fp | (myp & (S ? f.pa : f.pd) & pin_ok)) & f.theirs & tgt,
                [&](int to) { emit_pawn_sq(emit, to - CE, to, 0); });
    if (!f.checkers) {
        if (can_castle_k<S>(b, f.occ, f.threat)) emit(cmove(S ? 60 : 4, S ? 62 : 6, MF_KCASTLE), PC_KING);
        if (can_castle_q<S>(b, f.occ, f.threat)) emit(cmove(S ? 60 : 4, S ? 58 : 2, MF_QCASTLE), PC_KING);
    }
    // en passant: the rules of count_ep_ks
    if (b.p & 0xF0ull) {
        const u64 et = ep_target<S>(b);
        const u64 victim = S ? up(et) : down(et);
        const int to = lsb(et) & 63;
        u64 cand = (east1(victim) | west1(victim)) & myp;
        if (f.checkers) {
            cand = (victim == f.checkers) ? (cand & ~f.pinned) : 0ull;
            for (; cand; cand &= cand - 1) emit(cmove(lsb(cand), to, MF_EP));
        } else {
            const Sides<S> c(b);
            for (; cand; cand &= cand - 1)
                if (ep_legal<S>(c, f.pinned, lowbit(cand), et, victim)) emit(cmove(lsb(cand), to, MF_EP));
        }
    }
}

template <int S, class E> __device__ __forceinline__ void gen_leaf(const Pos& b, E& emit)
{
    gen_from_facts<S>(b, ks_facts<S>(b), emit);
}

// generateMovesOutOfCheck (MGB.h:2266-2463)
template <int S, class SL, class E>
__device__ __noinline__ void gen_evasions(const Pos& b, E& emit)
{
    const Sides<S> c(b);
    const u64 threat = threat_full<S, SL>(b, c);
    for (u64 s = king_set(c.king) & ~(threat | c.mine); s; s &= s - 1) emit(cmove(c.ksq, lsb(s), 0));
    const u64 att = checkers<S, SL>(b, c);
    if (!att || several(att)) return;
    const u64 pinned = find_pinned(c.ksq, c.tbq, c.trq, c.occ);
    const u64 safe = att | between_on(king_line(c.ksq, att), lsb(att), c.ksq);
    const u64 mine = c.mine & ~pinned;
    u64 tgt = ep_target<S>(b);
    const u64 victim = S ? up(tgt) : down(tgt);
    if (victim != att) tgt = 0;
    for (u64 pw = c.pawns & mine; pw; pw &= pw - 1) {
        const u64 p = lowbit(pw);
        const int from = lsb(p);
        const u64 d = push1<S>(p) & ~c.occ;
        if (d) {
            if (d & safe) {
                emit_pawn(emit, from, d, 0);
            } else {
                const u64 d2 = push1<S>(d & double_rank<S>()) & safe & ~c.occ;
                if (d2) emit(cmove(from, lsb(d2), MF_DOUBLE));
            }
        }
        const u64 caps = cap_w<S>(p) | cap_e<S>(p);
        const u64 hit = caps & c.theirs & safe;
        if (hit) emit_pawn(emit, from, hit, MF_CAPTURE);
        const u64 epd = caps & tgt;
        if (epd) emit(cmove(from, lsb(epd), MF_EP));
    }
    for (u64 s = b.n & mine; s; s &= s - 1)
        for (u64 m = __ldg(&g_knight[lsb(s)]) & safe; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), 0));
    for (u64 s = b.bq & mine; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & safe; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), 0));
    for (u64 s = b.rq & mine; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & safe; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), 0));
}

template <int S, class SL, class E>
__device__ __forceinline__ void gen_moves(const Pos& b, E& emit)
{
    const Sides<S> c(b);
    const u64 threat = threat_full<S, SL>(b, c);
    if (threat & c.king) {
        gen_evasions<S, SL>(b, emit);
        return;
    }
    const u64 pinned = find_pinned(c.ksq, c.tbq, c.trq, c.occ);
    auto capf = [&](u64 m) { return (lowbit(m) & c.theirs) ? MF_CAPTURE : 0; };
    for (u64 s = king_set(c.king) & ~(threat | c.mine); s; s &= s - 1) emit(cmove(c.ksq, lsb(s), capf(s)));
    for (u64 s = b.n & c.mine & ~pinned; s; s &= s - 1)
        for (u64 m = __ldg(&g_knight[lsb(s)]) & ~c.mine; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), capf(m)));
    const u64 my_bq = b.bq & c.mine, my_rq = b.rq & c.mine;
    for (u64 s = my_bq & pinned; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & ~c.mine & king_line(c.ksq, lowbit(s)); m; m &= m - 1)
            emit(cmove(lsb(s), lsb(m), capf(m)));
    for (u64 s = my_bq & ~pinned; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & ~c.mine; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), capf(m)));
    for (u64 s = my_rq & pinned; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & ~c.mine & king_line(c.ksq, lowbit(s)); m; m &= m - 1)
            emit(cmove(lsb(s), lsb(m), capf(m)));
    for (u64 s = my_rq & ~pinned; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & ~c.mine; m; m &= m - 1) emit(cmove(lsb(s), lsb(m), capf(m)));
    const u64 myp = c.pawns & c.mine;
    const u64 tgt = ep_target<S>(b);
    if (tgt) {
        const u64 victim = S ? up(tgt) : down(tgt);
        for (u64 s = (east1(victim) | west1(victim)) & myp; s; s &= s - 1)
            if (ep_legal<S>(c, pinned, lowbit(s), tgt, victim)) emit(cmove(lsb(s), lsb(tgt), MF_EP));
    }
    for (u64 s = myp & pinned; s; s &= s - 1) {
        const u64 p = lowbit(s);
        const int from = lsb(p);
        const u64 line = king_line(c.ksq, p);
        const u64 d = push1<S>(p) & line & ~c.occ;
        if (d) {
            emit(cmove(from, lsb(d), 0));
            const u64 d2 = push1<S>(d & double_rank<S>()) & ~c.occ;
            if (d2) emit(cmove(from, lsb(d2), MF_DOUBLE));
        }
        const u64 x = (cap_w<S>(p) & line) | (cap_e<S>(p) & line);
        if (x & c.theirs) emit_pawn(emit, from, x, MF_CAPTURE);
    }
    for (u64 s = myp & ~pinned; s; s &= s - 1) {
        const u64 p = lowbit(s);
        const int from = lsb(p);
        const u64 d = push1<S>(p) & ~c.occ;
        if (d) {
            emit_pawn(emit, from, d, 0);
            const u64 d2 = push1<S>(d & double_rank<S>()) & ~c.occ;
            if (d2) emit_pawn(emit, from, d2, MF_DOUBLE);
        }
        const u64 w = cap_w<S>(p) & c.theirs;
        if (w) emit_pawn(emit, from, w, MF_CAPTURE);
        const u64 e = cap_e<S>(p) & c.theirs;
        if (e) emit_pawn(emit, from, e, MF_CAPTURE);
    }
    if (can_castle_k<S>(b, c.occ, threat)) emit(cmove(S ? 60 : 4, S ? 62 : 6, MF_KCASTLE));
    if (can_castle_q<S>(b, c.occ, threat)) emit(cmove(S ? 60 : 4, S ? 58 : 2, MF_QCASTLE));
}

// ---------------------------------------------------------------------------
// makeMove
// ---------------------------------------------------------------------------

// updateCastleFlag (MGB.h:1302-1340)
__device__ __forceinline__ void castle_update(Pos& b, u64 sq, int mover)
{
    if (mover == 0) {
        if (sq & (1ull << 63)) set_bc(b, st_bc(b) & ~1);
        else if (sq & (1ull << 56)) set_bc(b, st_bc(b) & ~2);
    } else {
        if (sq & (1ull << 7)) set_wc(b, st_wc(b) & ~1);
        else if (sq & 1ull) set_wc(b, st_wc(b) & ~2);
    }
}

// makeMove<c,false> (MGB.h:3310-3570), en-passant file set only when an enemy
// pawn stands beside the pushed pawn (MGB.h:3528-3547)
template <int S>
__device__ __forceinline__ void make_move(Pos& b, u16 mv)
{
    const int from = mv & 63, to = (mv >> 6) & 63, fl = (mv >> 12) & 15;
    const u64 src = 1ull << from, dst = 1ull << to;
    // moving piece: K, N, P, Q, B else R; a promotion flag overrides
    const bool isK = b.k & src, isN = b.n & src, isP = (b.p & INNER) & src;
    const bool isB0 = b.bq & src, isR0 = b.rq & src;
    bool toN, toB, toR, toP;
    if (fl & 8) {
        const int pr = fl & 3;  // 0 N, 1 B, 2 R, 3 Q
        toN = pr == 0;
        toB = pr == 1 || pr == 3;
        toR = pr >= 2;
        toP = false;
    } else {
        toN = isN && !isK;
        toP = isP && !isK && !isN;
        const bool slider = !isK && !isN && !isP;
        toB = slider && isB0;                     // bishop or queen
        toR = slider && (isR0 || !isB0);          // rook, queen, or nothing
    }
    const bool pieceIsRook = (fl & 8) ? ((fl & 3) == 2) : (!isK && !isN && !isP && !(isB0 && isR0) && !isB0);
    const u64 clr = ~(src | dst);
    b.bq &= clr;
    b.rq &= clr;
    b.k &= clr;
    b.n &= clr;
    b.p &= ~((src | dst) & INNER);
    if (isK && !(fl & 8)) {
        b.k |= dst;
        if (S) set_bc(b, 0); else set_wc(b, 0);
    }
    if (toN) b.n |= dst;
    if (toP) b.p |= dst;
    if (toB) b.bq |= dst;
    if (toR) b.rq |= dst;
    b.w = S ? (b.w & ~dst) : ((b.w ^ src) | dst);
    if (fl == MF_EP) {
        const u64 victim = S ? up(dst) : down(dst);
        b.p &= ~(victim & INNER);
        if (S) b.w &= ~victim;
    }
    if (fl == MF_KCASTLE || fl == MF_QCASTLE) {
        const int base = S ? 56 : 0;
        const u64 rf = 1ull << (base + (fl == MF_KCASTLE ? 7 : 0));
        const u64 rt = 1ull << (base + (fl == MF_KCASTLE ? 5 : 3));
        b.rq = (b.rq ^ rf) | rt;
        if (!S) b.w = (b.w ^ rf) | rt;
    }
    set_side(b, 1 - S);
    set_ep(b, 0);
    castle_update(b, dst, S);
    if (pieceIsRook) castle_update(b, src, 1 - S);
    if (fl == MF_DOUBLE) {
        const u64 pawns = b.p & INNER;
        const u64 occ = b.k | pawns | b.n | b.bq | b.rq;
        const u64 enemy = S ? b.w : (occ & ~b.w);
        if ((east1(dst) | west1(dst)) & pawns & enemy) set_ep(b, (from & 7) + 1);
    }
}

// the bit of square s (0..63) from two 32-bit shifts: PTX clamps a shift
// amount of 32 or more to 32, which clears the word, so the half that does
// not hold the square is 0 with no select (0.2-0.3% less leaf time than the
// 64-bit variable shift)
__device__ __forceinline__ u64 bit64(u32 s)
{
    u32 lo, hi;
    asm("shl.b32 %0, %1, %2;" : "=r"(lo) : "r"(1u), "r"(s));
    asm("shl.b32 %0, %1, %2;" : "=r"(hi) : "r"(1u), "r"(s - 32u));
    return ((u64)hi << 32) | lo;
}

// makeMove for a child whose moves are only counted: it writes what the count
// for the side to move next reads (the pieces, that side's castling rights
// and the exact en-passant file, as make_move) and leaves the mover's own
// castling rights and the side bit as they were.  `piece` is the moving piece
// that lands on the target square (PC_*; the promoted piece for a
// promotion), so nothing is looked up on the board or decoded from the flags,
// plus PC_EP_FLAG on a double push that gives the opponent an en-passant
// capture.
template <int S>
__device__ __forceinline__ void make_child(Pos& b, u16 mv, u32 piece)
{
    const int from = mv & 63, to = (mv >> 6) & 63, fl = (mv >> 12) & 15;
    const u64 src = bit64((u32)from), dst = bit64((u32)to);
    const u32 pc = piece & 7u;
    const bool toN = pc == PC_KNIGHT;
    const bool toB = pc == PC_BISHOP || pc == PC_QUEEN;
    const bool toR = pc == PC_ROOK || pc == PC_QUEEN;
    const bool toP = pc == PC_PAWN;
    const u64 clr = ~(src | dst);
    b.bq = (b.bq & clr) | (toB ? dst : 0ull);
    b.rq = (b.rq & clr) | (toR ? dst : 0ull);
    b.n = (b.n & clr) | (toN ? dst : 0ull);
    b.p = (b.p & ~((src | dst) & INNER)) | (toP ? dst : 0ull);
    if (pc == PC_KING) b.k = (b.k ^ src) | dst;
    b.w = S ? (b.w & ~dst) : ((b.w ^ src) | dst);
    if (fl == MF_EP) {
        const u64 victim = S ? up(dst) : down(dst);
        b.p &= ~(victim & INNER);
        if (S) b.w &= ~victim;
    }
    if (fl == MF_KCASTLE || fl == MF_QCASTLE) {
        const int base = S ? 56 : 0;
        const u64 rf = 1ull << (base + (fl == MF_KCASTLE ? 7 : 0));
        const u64 rt = 1ull << (base + (fl == MF_KCASTLE ? 5 : 3));
        b.rq = (b.rq ^ rf) | rt;
        if (!S) b.w = (b.w ^ rf) | rt;
    }
    set_ep(b, 0);
    // a move onto the other side's rook corner takes that side's right
    // (updateCastleFlag, MGB.h:1310-1340): h8/a8 clear black's bits 2/3,
    // h1/a1 clear white's bits 0/1
    b.p &= S ? ~(((dst >> 7) & 1ull) | ((dst << 1) & 2ull)) : ~(((dst >> 61) & 4ull) | ((dst >> 53) & 8ull));
    if (piece & PC_EP_FLAG) set_ep(b, (from & 7) + 1);
}

// ---------------------------------------------------------------------------
// generateBoards (reference order, reference child-board bytes)
// ---------------------------------------------------------------------------

__device__ __forceinline__ u64 new_white(const Pos& b, int S, u64 src, u64 dst)
{
    return S ? (b.w & ~dst) : ((b.w ^ src) | dst);
}

// addSlidingMove (MGB.h:1342-1397)
template <int S, class E> __device__ __forceinline__ void bd_slider(E& emit, const Pos& b, u64 src, u64 dst)
{
    Pos nb;
    nb.bq = b.bq & ~dst;
    nb.rq = b.rq & ~dst;
    nb.k = b.k & ~dst;
    nb.n = b.n & ~dst;
    nb.p = b.p & ~(dst & INNER);
    const u64 isb = nb.bq & src, isr = nb.rq & src;
    nb.bq ^= isb;
    nb.rq ^= isr;
    if (isb) nb.bq |= dst;
    if (isr) nb.rq |= dst;
    nb.w = new_white(b, S, src, dst);
    set_side(nb, 1 - S);
    set_ep(nb, 0);
    castle_update(nb, dst, S);
    castle_update(nb, src, 1 - S);
    emit(nb);
}
// addKnightMove (MGB.h:1400-1438)
template <int S, class E> __device__ __forceinline__ void bd_knight(E& emit, const Pos& b, u64 src, u64 dst)
{
    Pos nb;
    nb.bq = b.bq & ~dst;
    nb.rq = b.rq & ~dst;
    nb.k = b.k & ~dst;
    nb.p = b.p & ~(dst & INNER);
    nb.n = (b.n ^ src) | dst;
    nb.w = new_white(b, S, src, dst);
    set_side(nb, 1 - S);
    set_ep(nb, 0);
    castle_update(nb, dst, S);
    emit(nb);
}
// addKingMove (MGB.h:1441-1484)
template <int S, class E> __device__ __forceinline__ void bd_king(E& emit, const Pos& b, u64 src, u64 dst)
{
    Pos nb;
    nb.bq = b.bq & ~dst;
    nb.rq = b.rq & ~dst;
    nb.n = b.n & ~dst;
    nb.p = b.p & ~(dst & INNER);
    nb.k = (b.k ^ src) | dst;
    nb.w = new_white(b, S, src, dst);
    if (S) set_bc(nb, 0); else set_wc(nb, 0);
    set_side(nb, 1 - S);
    set_ep(nb, 0);
    castle_update(nb, dst, S);
    emit(nb);
}
// addCastleMove (MGB.h:1487-1522)
template <int S, class E> __device__ __forceinline__ void bd_castle(E& emit, const Pos& b, bool kingside)
{
    const int base = S ? 56 : 0;
    const u64 kf = 1ull << (base + 4), kt = 1ull << (base + (kingside ? 6 : 2));
    const u64 rf = 1ull << (base + (kingside ? 7 : 0)), rt = 1ull << (base + (kingside ? 5 : 3));
    Pos nb;
    nb.bq = b.bq;
    nb.p = b.p;
    nb.n = b.n;
    nb.k = (b.k ^ kf) | kt;
    nb.rq = (b.rq ^ rf) | rt;
    set_side(nb, 1 - S);
    set_ep(nb, 0);
    set_hm(nb, 0);
    if (S == 0) {
        nb.w = (b.w ^ (kf | rf)) | (kt | rt);
        set_wc(nb, 0);
    } else {
        set_bc(nb, 0);
        nb.w = b.w;
    }
    emit(nb);
}
// addSinglePawnMove (MGB.h:1527-1574)
template <int S, class E> __device__ __forceinline__ void bd_step(E& emit, const Pos& b, u64 src, u64 dst, bool dbl, int from)
{
    Pos nb;
    nb.bq = b.bq & ~dst;
    nb.rq = b.rq & ~dst;
    nb.n = b.n & ~dst;
    nb.k = b.k;
    nb.p = (b.p ^ src) | dst;
    nb.w = new_white(b, S, src, dst);
    set_side(nb, 1 - S);
    set_ep(nb, dbl ? (from & 7) + 1 : 0);
    set_hm(nb, 0);
    emit(nb);
}
// addEnPassentMove (MGB.h:1576-1618)
template <int S, class E> __device__ __forceinline__ void bd_ep(E& emit, const Pos& b, u64 src, u64 dst)
{
    const u64 victim = S ? up(dst) : down(dst);
    Pos nb;
    nb.bq = b.bq;
    nb.rq = b.rq;
    nb.n = b.n;
    nb.k = b.k;
    nb.p = (b.p ^ (victim | src)) | dst;
    nb.w = S ? (b.w ^ victim) : ((b.w ^ src) | dst);
    set_side(nb, 1 - S);
    set_hm(nb, 0);
    set_ep(nb, 0);
    emit(nb);
}
// addPawnMoves (MGB.h:1622-1699): promotions N, B, Q, R
template <int S, class E> __device__ __forceinline__ void bd_pawn(E& emit, const Pos& b, u64 src, u64 dst)
{
    if (!(dst & BACK_RANKS)) {
        bd_step<S>(emit, b, src, dst, false, 0);
        return;
    }
    Pos nb;
    nb.k = b.k;
    nb.w = new_white(b, S, src, dst);
    nb.p = b.p ^ src;
    set_side(nb, 1 - S);
    set_ep(nb, 0);
    set_hm(nb, 0);
    castle_update(nb, dst, S);
    nb.n = b.n | dst;
    nb.bq = b.bq & ~dst;
    nb.rq = b.rq & ~dst;
    emit(nb);
    nb.n = b.n & ~dst;
    nb.bq = b.bq | dst;
    nb.rq = b.rq & ~dst;
    emit(nb);
    nb.rq = b.rq | dst;
    emit(nb);
    nb.bq = b.bq & ~dst;
    emit(nb);
}

template <int S, class SL, class E>
__device__ __noinline__ void gen_boards_evasions(const Pos& b, E& emit)
{
    const Sides<S> c(b);
    const u64 threat = threat_full<S, SL>(b, c);
    for (u64 s = king_set(c.king) & ~(threat | c.mine); s; s &= s - 1) bd_king<S>(emit, b, c.king, lowbit(s));
    const u64 att = checkers<S, SL>(b, c);
    if (!att || several(att)) return;
    const u64 pinned = find_pinned(c.ksq, c.tbq, c.trq, c.occ);
    const u64 safe = att | between_on(king_line(c.ksq, att), lsb(att), c.ksq);
    const u64 mine = c.mine & ~pinned;
    u64 tgt = ep_target<S>(b);
    const u64 victim = S ? up(tgt) : down(tgt);
    if (victim != att) tgt = 0;
    for (u64 pw = c.pawns & mine; pw; pw &= pw - 1) {
        const u64 p = lowbit(pw);
        const u64 d = push1<S>(p) & ~c.occ;
        if (d) {
            if (d & safe) {
                bd_pawn<S>(emit, b, p, d);
            } else {
                const u64 d2 = push1<S>(d & double_rank<S>()) & safe & ~c.occ;
                if (d2) bd_step<S>(emit, b, p, d2, true, lsb(p));
            }
        }
        const u64 caps = cap_w<S>(p) | cap_e<S>(p);
        const u64 hit = caps & c.theirs & safe;
        if (hit) bd_pawn<S>(emit, b, p, hit);
        const u64 epd = caps & tgt;
        if (epd) bd_ep<S>(emit, b, p, epd);
    }
    for (u64 s = b.n & mine; s; s &= s - 1)
        for (u64 m = __ldg(&g_knight[lsb(s)]) & safe; m; m &= m - 1) bd_knight<S>(emit, b, lowbit(s), lowbit(m));
    for (u64 s = b.bq & mine; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & safe; m; m &= m - 1) bd_slider<S>(emit, b, lowbit(s), lowbit(m));
    for (u64 s = b.rq & mine; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & safe; m; m &= m - 1) bd_slider<S>(emit, b, lowbit(s), lowbit(m));
}

template <int S, class SL, class E>
__device__ __forceinline__ void gen_boards(const Pos& b, E& emit)
{
    const Sides<S> c(b);
    const u64 threat = threat_full<S, SL>(b, c);
    if (threat & c.king) {
        gen_boards_evasions<S, SL>(b, emit);
        return;
    }
    const u64 pinned = find_pinned(c.ksq, c.tbq, c.trq, c.occ);
    const u64 myp = c.pawns & c.mine;
    const u64 tgt = ep_target<S>(b);
    if (tgt) {
        const u64 victim = S ? up(tgt) : down(tgt);
        for (u64 s = (east1(victim) | west1(victim)) & myp; s; s &= s - 1)
            if (ep_legal<S>(c, pinned, lowbit(s), tgt, victim)) bd_ep<S>(emit, b, lowbit(s), tgt);
    }
    for (u64 s = myp & pinned; s; s &= s - 1) {
        const u64 p = lowbit(s);
        const int from = lsb(p);
        const u64 line = king_line(c.ksq, p);
        const u64 d = push1<S>(p) & line & ~c.occ;
        if (d) {
            bd_step<S>(emit, b, p, d, false, from);
            const u64 d2 = push1<S>(d & double_rank<S>()) & ~c.occ;
            if (d2) bd_step<S>(emit, b, p, d2, true, from);
        }
        const u64 x = (cap_w<S>(p) & line) | (cap_e<S>(p) & line);
        if (x & c.theirs) bd_pawn<S>(emit, b, p, x);
    }
    for (u64 s = myp & ~pinned; s; s &= s - 1) {
        const u64 p = lowbit(s);
        const u64 d = push1<S>(p) & ~c.occ;
        if (d) {
            bd_pawn<S>(emit, b, p, d);
            const u64 d2 = push1<S>(d & double_rank<S>()) & ~c.occ;
            if (d2) bd_step<S>(emit, b, p, d2, true, lsb(p));
        }
        const u64 w = cap_w<S>(p) & c.theirs;
        if (w) bd_pawn<S>(emit, b, p, w);
        const u64 e = cap_e<S>(p) & c.theirs;
        if (e) bd_pawn<S>(emit, b, p, e);
    }
    if (can_castle_k<S>(b, c.occ, threat)) bd_castle<S>(emit, b, true);
    if (can_castle_q<S>(b, c.occ, threat)) bd_castle<S>(emit, b, false);
    for (u64 s = king_set(c.king) & ~(threat | c.mine); s; s &= s - 1) bd_king<S>(emit, b, c.king, lowbit(s));
    for (u64 s = b.n & c.mine & ~pinned; s; s &= s - 1)
        for (u64 m = __ldg(&g_knight[lsb(s)]) & ~c.mine; m; m &= m - 1) bd_knight<S>(emit, b, lowbit(s), lowbit(m));
    const u64 my_bq = b.bq & c.mine, my_rq = b.rq & c.mine;
    for (u64 s = my_bq & pinned; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & ~c.mine & king_line(c.ksq, lowbit(s)); m; m &= m - 1)
            bd_slider<S>(emit, b, lowbit(s), lowbit(m));
    for (u64 s = my_bq & ~pinned; s; s &= s - 1)
        for (u64 m = SL::bishop(lsb(s), c.occ) & ~c.mine; m; m &= m - 1) bd_slider<S>(emit, b, lowbit(s), lowbit(m));
    for (u64 s = my_rq & pinned; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & ~c.mine & king_line(c.ksq, lowbit(s)); m; m &= m - 1)
            bd_slider<S>(emit, b, lowbit(s), lowbit(m));
    for (u64 s = my_rq & ~pinned; s; s &= s - 1)
        for (u64 m = SL::rook(lsb(s), c.occ) & ~c.mine; m; m &= m - 1) bd_slider<S>(emit, b, lowbit(s), lowbit(m));
}

}  // namespace pg
