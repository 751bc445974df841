/*
 * oracle.c -- CPU restatement of the reference perft move generator.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  The product never uses this file.
 *
 * Citations are file:line into the reference project sarona-RD/perft_gpu.
 * "MGB.h" below is its MoveGeneratorBitboard.h.  The legality rules, the move
 * order of generateMoves / generateBoards and the state updates of makeMove
 * are the reference's and are kept exactly, including its quirks:
 *   - castling checks only the flag, the empty squares and the unattacked
 *     squares, not that the rook is there (MGB.h:3200-3237);
 *   - in check, en passant is allowed only when the captured pawn is the
 *     single checker (MGB.h:2903-2906);
 *   - pinned pieces never answer a check (MGB.h:2878-2880);
 *   - a pinned pawn's push never expands into promotions (MGB.h:3123-3135);
 *   - makeMove sets the en-passant file only when an enemy pawn stands beside
 *     the pushed pawn (MGB.h:3528-3547, EXACT_EN_PASSENT_FLAGGING).
 * Bit manipulation uses only portable GCC builtins (x86 and Arm alike).
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef uint64_t u64;
typedef uint32_t u32;

#define BB(sq) (1ull << (sq))

static const u64 FILE_A = 0x0101010101010101ull;
static const u64 FILE_H = 0x8080808080808080ull;
static const u64 RANK_1 = 0x00000000000000FFull;
static const u64 RANK_3 = 0x0000000000FF0000ull;
static const u64 RANK_8 = 0xFF00000000000000ull;
static const u64 INNER_RANKS = 0x00FFFFFFFFFFFF00ull; /* ranks 2..7 */

/* castling square sets (MGB.h:43-55) */
static const u64 W_KS_PATH = 0x60ull;                /* f1 g1 */
static const u64 W_QS_SAFE = 0x0Cull;                /* c1 d1 */
static const u64 W_QS_PATH = 0x0Eull;                /* b1 c1 d1 */
static const u64 B_KS_PATH = 0x6000000000000000ull;  /* f8 g8 */
static const u64 B_QS_SAFE = 0x0C00000000000000ull;  /* c8 d8 */
static const u64 B_QS_PATH = 0x0E00000000000000ull;  /* b8 c8 d8 */

/* move flags (chess.h:272-293) */
enum { F_QUIET = 0, F_DOUBLE = 1, F_KCASTLE = 2, F_QCASTLE = 3, F_CAPTURE = 4,
       F_EP = 5, F_PROMO_N = 8, F_PROMO_B = 9, F_PROMO_R = 10, F_PROMO_Q = 11 };

static inline int lsb(u64 x) { return __builtin_ctzll(x); }
static inline int popc(u64 x) { return __builtin_popcountll(x); }
static inline int several(u64 x) { return (x & (x - 1)) != 0; }

/* ---- packed game state in the pawns word (chess.h:211-226) ---- */
static inline int st_wcastle(const or_board *b) { return (int)(b->pawns & 3); }
static inline int st_bcastle(const or_board *b) { return (int)((b->pawns >> 2) & 3); }
static inline int st_ep(const or_board *b) { return (int)((b->pawns >> 4) & 15); }
static inline int st_side(const or_board *b) { return (int)(b->pawns >> 63); }
static inline void set_wcastle(or_board *b, int v) { b->pawns = (b->pawns & ~3ull) | (u64)(v & 3); }
static inline void set_bcastle(or_board *b, int v) { b->pawns = (b->pawns & ~12ull) | ((u64)(v & 3) << 2); }
static inline void set_ep(or_board *b, int v) { b->pawns = (b->pawns & ~0xF0ull) | ((u64)(v & 15) << 4); }
static inline void set_side(or_board *b, int v) { b->pawns = (b->pawns & ~(1ull << 63)) | ((u64)(v & 1) << 63); }
static inline void set_halfmove(or_board *b, int v) { b->pawns = (b->pawns & ~(0x7Full << 56)) | ((u64)(v & 0x7F) << 56); }

/* ---- one-step shifts (MGB.h:455-493) ---- */
static inline u64 up(u64 x) { return x << 8; }
static inline u64 down(u64 x) { return x >> 8; }
static inline u64 right1(u64 x) { return (x << 1) & ~FILE_A; }
static inline u64 left1(u64 x) { return (x >> 1) & ~FILE_H; }
static inline u64 up_right(u64 x) { return (x << 9) & ~FILE_A; }
static inline u64 up_left(u64 x) { return (x << 7) & ~FILE_H; }
static inline u64 down_right(u64 x) { return (x >> 7) & ~FILE_A; }
static inline u64 down_left(u64 x) { return (x >> 9) & ~FILE_H; }

/* ---- occluded fills, Kogge-Stone (MGB.h:504-728) ----
 * gen: slider set, pro: squares a ray may pass through.  Returns the squares
 * attacked in one direction (first blocker included). */
static inline u64 ray_up_shift(u64 gen, u64 pro, int s, u64 keep)
{
    pro &= keep;
    gen |= pro & (gen << s);
    pro &= pro << s;
    gen |= pro & (gen << (2 * s));
    pro &= pro << (2 * s);
    gen |= pro & (gen << (4 * s));
    return (gen << s) & keep;
}
static inline u64 ray_down_shift(u64 gen, u64 pro, int s, u64 keep)
{
    pro &= keep;
    gen |= pro & (gen >> s);
    pro &= pro >> s;
    gen |= pro & (gen >> (2 * s));
    pro &= pro >> (2 * s);
    gen |= pro & (gen >> (4 * s));
    return (gen >> s) & keep;
}
static inline u64 ks_north(u64 g, u64 p) { return ray_up_shift(g, p, 8, ~0ull); }
static inline u64 ks_south(u64 g, u64 p) { return ray_down_shift(g, p, 8, ~0ull); }
static inline u64 ks_east(u64 g, u64 p) { return ray_up_shift(g, p, 1, ~FILE_A); }
static inline u64 ks_west(u64 g, u64 p) { return ray_down_shift(g, p, 1, ~FILE_H); }
static inline u64 ks_ne(u64 g, u64 p) { return ray_up_shift(g, p, 9, ~FILE_A); }
static inline u64 ks_nw(u64 g, u64 p) { return ray_up_shift(g, p, 7, ~FILE_H); }
static inline u64 ks_se(u64 g, u64 p) { return ray_down_shift(g, p, 7, ~FILE_A); }
static inline u64 ks_sw(u64 g, u64 p) { return ray_down_shift(g, p, 9, ~FILE_H); }

static inline u64 ks_bishop(u64 g, u64 p) { return ks_ne(g, p) | ks_nw(g, p) | ks_se(g, p) | ks_sw(g, p); }
static inline u64 ks_rook(u64 g, u64 p) { return ks_north(g, p) | ks_south(g, p) | ks_east(g, p) | ks_west(g, p); }

/* knight and king patterns, set-wise (MGB.h:845-866) */
static u64 knight_set(u64 n)
{
    u64 a = ((n >> 1) & ~FILE_H) | ((n << 1) & ~FILE_A);
    u64 b = ((n >> 2) & 0x3F3F3F3F3F3F3F3Full) | ((n << 2) & 0xFCFCFCFCFCFCFCFCull);
    return (a << 16) | (a >> 16) | (b << 8) | (b >> 8);
}
static u64 king_set(u64 k)
{
    u64 a = right1(k) | left1(k);
    u64 row = k | a;
    return a | up(row) | down(row);
}

/* ---- tables (MGB.h:982-1076) ---- */
static u64 T_KNIGHT[64], T_KING[64], T_ROOK_RAY[64], T_BISHOP_RAY[64];
static u64 T_BETWEEN[64][64], T_LINE[64][64];
static int g_slider_mode = 1;

/* fancy magics: own search, own tables (the values differ from the
 * reference's fixed-shift factors; the attack sets they return are equal) */
typedef struct { u64 mask, magic; u64 *table; int shift; } magic_entry;
static magic_entry M_ROOK[64], M_BISHOP[64];
static u64 magic_store[102400 + 5248];

static u64 slow_rays(int sq, u64 occ, int rook)
{
    static const int rd[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
    static const int bd[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
    const int (*d)[2] = rook ? rd : bd;
    u64 att = 0;
    for (int k = 0; k < 4; k++) {
        int r = sq >> 3, f = sq & 7;
        for (;;) {
            r += d[k][0]; f += d[k][1];
            if (r < 0 || r > 7 || f < 0 || f > 7) break;
            att |= BB(r * 8 + f);
            if (occ & BB(r * 8 + f)) break;
        }
    }
    return att;
}

static u64 xs_state = 0x2545F4914F6CDD1Dull;
static u64 xs_next(void)
{
    xs_state ^= xs_state >> 12;
    xs_state ^= xs_state << 25;
    xs_state ^= xs_state >> 27;
    return xs_state * 0x2545F4914F6CDD1Dull;
}

static u64 *build_magic(magic_entry *e, int sq, int rook, u64 *store)
{
    u64 edges = ((RANK_1 | RANK_8) & ~(RANK_1 << (8 * (sq >> 3)))) |
                ((FILE_A | FILE_H) & ~(FILE_A << (sq & 7)));
    u64 mask = slow_rays(sq, 0, rook) & ~edges;
    int bits = popc(mask);
    int size = 1 << bits;
    u64 occ[4096], att[4096];
    int used_epoch[4096];
    int n = 0;
    u64 sub = 0;
    do { /* carry-rippler enumeration of the subsets of mask */
        occ[n] = sub;
        att[n] = slow_rays(sq, sub, rook);
        n++;
        sub = (sub - mask) & mask;
    } while (sub);
    for (int i = 0; i < size; i++) used_epoch[i] = -1;
    e->mask = mask;
    e->shift = 64 - bits;
    e->table = store;
    for (int attempt = 0;; attempt++) {
        u64 m = xs_next() & xs_next() & xs_next();
        if (popc((mask * m) & 0xFF00000000000000ull) < 6) continue;
        int ok = 1;
        for (int i = 0; i < n && ok; i++) {
            int idx = (int)((occ[i] * m) >> e->shift);
            if (used_epoch[idx] != attempt) {
                used_epoch[idx] = attempt;
                store[idx] = att[i];
            } else if (store[idx] != att[i]) {
                ok = 0;
            }
        }
        if (ok) { e->magic = m; break; }
    }
    return store + size;
}

static inline u64 rook_att_sq(int sq, u64 occ)
{
    const magic_entry *e = &M_ROOK[sq];
    return e->table[((occ & e->mask) * e->magic) >> e->shift];
}
static inline u64 bishop_att_sq(int sq, u64 occ)
{
    const magic_entry *e = &M_BISHOP[sq];
    return e->table[((occ & e->mask) * e->magic) >> e->shift];
}

/* bishopAttacks / rookAttacks for one piece (MGB.h:732-803); pro = squares
 * the ray may cross. */
static inline u64 bishop_one(u64 piece, u64 pro)
{
    return g_slider_mode ? bishop_att_sq(lsb(piece), ~pro) : ks_bishop(piece, pro);
}
static inline u64 rook_one(u64 piece, u64 pro)
{
    return g_slider_mode ? rook_att_sq(lsb(piece), ~pro) : ks_rook(piece, pro);
}
/* multiBishopAttacks / multiRookAttacks (MGB.h:805-829) */
static inline u64 bishop_many(u64 set, u64 pro)
{
    if (!g_slider_mode) return ks_bishop(set, pro);
    u64 a = 0;
    for (; set; set &= set - 1) a |= bishop_att_sq(lsb(set), ~pro);
    return a;
}
static inline u64 rook_many(u64 set, u64 pro)
{
    if (!g_slider_mode) return ks_rook(set, pro);
    u64 a = 0;
    for (; set; set &= set - 1) a |= rook_att_sq(lsb(set), ~pro);
    return a;
}

static int g_ready = 0;
static pthread_mutex_t g_init_lock = PTHREAD_MUTEX_INITIALIZER;

void or_init(int slider_mode)
{
    pthread_mutex_lock(&g_init_lock);
    g_slider_mode = slider_mode ? 1 : 0;
    if (!g_ready) {
        for (int s = 0; s < 64; s++) {
            T_KNIGHT[s] = knight_set(BB(s));
            T_KING[s] = king_set(BB(s));
            T_ROOK_RAY[s] = slow_rays(s, 0, 1);
            T_BISHOP_RAY[s] = slow_rays(s, 0, 0);
        }
        /* Between / Line (MGB.h:1012-1021): squares strictly between two
         * aligned squares, and the whole line through them. */
        for (int a = 0; a < 64; a++)
            for (int b = 0; b < 64; b++) {
                T_BETWEEN[a][b] = 0;
                T_LINE[a][b] = 0;
                if (a == b) continue;
                int rook = (T_ROOK_RAY[a] & BB(b)) != 0;
                int bishop = (T_BISHOP_RAY[a] & BB(b)) != 0;
                if (!rook && !bishop) continue;
                T_BETWEEN[a][b] = slow_rays(a, BB(b), rook) & slow_rays(b, BB(a), rook);
                T_LINE[a][b] = (slow_rays(a, 0, rook) & slow_rays(b, 0, rook)) | BB(a) | BB(b);
            }
        u64 *p = magic_store;
        for (int s = 0; s < 64; s++) p = build_magic(&M_ROOK[s], s, 1, p);
        for (int s = 0; s < 64; s++) p = build_magic(&M_BISHOP[s], s, 0, p);
        g_ready = 1;
    }
    pthread_mutex_unlock(&g_init_lock);
}

/* ---- per-position facts shared by count / generate ---- */
typedef struct {
    int side, ksq;
    u64 pawns, occ, mine, theirs, their_bq, their_rq, king, pinned, threat;
} ctx_t;

/* findPinnedPieces (MGB.h:1213-1249): an own or enemy piece that is the only
 * piece between the king and an aligned enemy slider. */
static u64 find_pinned(int ksq, u64 their_bq, u64 their_rq, u64 occ)
{
    u64 cand = (T_BISHOP_RAY[ksq] & their_bq) | (T_ROOK_RAY[ksq] & their_rq);
    u64 pinned = 0;
    for (; cand; cand &= cand - 1) {
        u64 inb = T_BETWEEN[lsb(cand)][ksq] & occ;
        if (!several(inb)) pinned |= inb;
    }
    return pinned;
}

/* findAttackedSquares (MGB.h:1254-1298): squares the enemy attacks with the
 * moving side's king taken off the board. */
static u64 find_threat(const or_board *b, const ctx_t *c)
{
    u64 pro = ~c->occ | c->king;
    u64 tp = c->pawns & c->theirs;
    u64 t = c->side ? (up_right(tp) | up_left(tp)) : (down_right(tp) | down_left(tp));
    t |= knight_set(b->knights & c->theirs);
    t |= bishop_many(c->their_bq, pro);
    t |= rook_many(c->their_rq, pro);
    t |= king_set(b->kings & c->theirs);
    return t;
}

static void ctx_init(ctx_t *c, const or_board *b)
{
    c->side = st_side(b);
    c->pawns = b->pawns & INNER_RANKS;
    c->occ = b->kings | c->pawns | b->knights | b->bishop_queens | b->rook_queens;
    u64 black = c->occ & ~b->white;
    c->mine = c->side ? black : b->white;
    c->theirs = c->side ? b->white : black;
    c->their_bq = b->bishop_queens & c->theirs;
    c->their_rq = b->rook_queens & c->theirs;
    c->king = b->kings & c->mine;
    c->ksq = c->king ? lsb(c->king) : 0;
    c->pinned = find_pinned(c->ksq, c->their_bq, c->their_rq, c->occ);
    c->threat = find_threat(b, c);
}

static inline u64 push1(int side, u64 x) { return side ? down(x) : up(x); }
static inline u64 cap_west(int side, u64 x) { return side ? down_left(x) : up_left(x); }
static inline u64 cap_east(int side, u64 x) { return side ? down_right(x) : up_right(x); }
static inline u64 double_rank(int side) { return RANK_3 << (side * 24); }
static inline u64 ep_target(const or_board *b, int side)
{
    int ep = st_ep(b);
    if (!ep) return 0;
    return BB(ep - 1) << (side ? 16 : 40);
}

/* single checker set (MGB.h:2842-2860) */
static u64 checkers(const or_board *b, const ctx_t *c)
{
    u64 k = c->king;
    u64 a = (c->side ? (down_right(k) | down_left(k)) : (up_right(k) | up_left(k))) &
            (c->pawns & c->theirs);
    a |= knight_set(k) & (b->knights & c->theirs);
    a |= bishop_one(k, ~c->occ) & c->their_bq;
    a |= rook_one(k, ~c->occ) & c->their_rq;
    return a;
}

/* ======================= countMoves ======================= */

/* countMovesOutOfCheck (MGB.h:2825-3002) */
static u32 count_evasions(const or_board *b, const ctx_t *c)
{
    u32 n = (u32)popc(T_KING[c->ksq] & ~(c->threat | c->mine));
    u64 att = checkers(b, c);
    if (several(att) || !att) return n;
    int side = c->side;
    u64 safe = att | T_BETWEEN[c->ksq][lsb(att)];
    u64 mine = c->mine & ~c->pinned;
    u64 tgt = ep_target(b, side);
    u64 victim = side ? up(tgt) : down(tgt);
    if (victim != att) tgt = 0;
    for (u64 pw = c->pawns & mine; pw; pw &= pw - 1) {
        u64 p = pw & (0 - pw);
        u64 d = push1(side, p) & ~c->occ;
        if (d) {
            if (d & safe) {
                n += (d & (RANK_1 | RANK_8)) ? 4 : 1;
            } else if (push1(side, d & double_rank(side)) & safe & ~c->occ) {
                n++;
            }
        }
        u64 caps = (cap_west(side, p) | cap_east(side, p));
        u64 hit = caps & c->theirs & safe;
        if (hit) n += (hit & (RANK_1 | RANK_8)) ? 4 : 1;
        if (caps & tgt) n++;
    }
    for (u64 s = b->knights & mine; s; s &= s - 1) n += popc(T_KNIGHT[lsb(s)] & safe);
    for (u64 s = b->bishop_queens & mine; s; s &= s - 1)
        n += popc(bishop_one(s & (0 - s), ~c->occ) & safe);
    for (u64 s = b->rook_queens & mine; s; s &= s - 1)
        n += popc(rook_one(s & (0 - s), ~c->occ) & safe);
    return n;
}

/* en-passant legality outside check (MGB.h:3058-3093) */
static int ep_ok(const ctx_t *c, u64 pawn, u64 tgt, u64 victim)
{
    if (pawn & c->pinned) return (tgt & T_LINE[lsb(pawn)][c->ksq]) != 0;
    u64 pro = ~c->occ | victim | pawn;
    return ((ks_east(c->their_rq, pro) | ks_west(c->their_rq, pro)) & c->king) == 0;
}

static int castle_ks_ok(const or_board *b, const ctx_t *c)
{
    if (c->side == 0)
        return (st_wcastle(b) & 1) && !(W_KS_PATH & c->occ) && !(W_KS_PATH & c->threat);
    return (st_bcastle(b) & 1) && !(B_KS_PATH & c->occ) && !(B_KS_PATH & c->threat);
}
static int castle_qs_ok(const or_board *b, const ctx_t *c)
{
    if (c->side == 0)
        return (st_wcastle(b) & 2) && !(W_QS_PATH & c->occ) && !(W_QS_SAFE & c->threat);
    return (st_bcastle(b) & 2) && !(B_QS_PATH & c->occ) && !(B_QS_SAFE & c->threat);
}

/* countMoves (MGB.h:3008-3295) */
static u32 count_ctx(const or_board *b, const ctx_t *c)
{
    if (c->threat & c->king) return count_evasions(b, c);
    int side = c->side;
    u32 n = 0;
    u64 my_pawns = c->pawns & c->mine;
    u64 tgt = ep_target(b, side);
    if (tgt) {
        u64 victim = side ? up(tgt) : down(tgt);
        for (u64 s = (right1(victim) | left1(victim)) & my_pawns; s; s &= s - 1)
            n += (u32)ep_ok(c, s & (0 - s), tgt, victim);
    }
    for (u64 s = my_pawns & c->pinned; s; s &= s - 1) {
        u64 p = s & (0 - s);
        u64 line = T_LINE[lsb(p)][c->ksq];
        u64 d = push1(side, p) & line & ~c->occ;
        if (d) {
            n++;
            if (push1(side, d & double_rank(side)) & ~c->occ) n++;
        }
        u64 x = (cap_west(side, p) & line) | (cap_east(side, p) & line);
        if (x & c->theirs) n += (x & (RANK_1 | RANK_8)) ? 4 : 1;
    }
    u64 free_pawns = my_pawns & ~c->pinned;
    u64 d = push1(side, free_pawns) & ~c->occ;
    n += popc(d) + 3 * popc(d & (RANK_1 | RANK_8));
    n += popc(push1(side, d & double_rank(side)) & ~c->occ);
    u64 w = cap_west(side, free_pawns) & c->theirs;
    n += popc(w) + 3 * popc(w & (RANK_1 | RANK_8));
    u64 e = cap_east(side, free_pawns) & c->theirs;
    n += popc(e) + 3 * popc(e & (RANK_1 | RANK_8));
    n += (u32)castle_ks_ok(b, c) + (u32)castle_qs_ok(b, c);
    n += popc(T_KING[c->ksq] & ~(c->threat | c->mine));
    for (u64 s = b->knights & c->mine & ~c->pinned; s; s &= s - 1)
        n += popc(T_KNIGHT[lsb(s)] & ~c->mine);
    u64 my_bq = b->bishop_queens & c->mine, my_rq = b->rook_queens & c->mine;
    for (u64 s = my_bq & c->pinned; s; s &= s - 1)
        n += popc(bishop_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]);
    for (u64 s = my_bq & ~c->pinned; s; s &= s - 1)
        n += popc(bishop_one(s & (0 - s), ~c->occ) & ~c->mine);
    for (u64 s = my_rq & c->pinned; s; s &= s - 1)
        n += popc(rook_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]);
    for (u64 s = my_rq & ~c->pinned; s; s &= s - 1)
        n += popc(rook_one(s & (0 - s), ~c->occ) & ~c->mine);
    return n;
}

uint32_t or_count_moves(const or_board *b)
{
    ctx_t c;
    ctx_init(&c, b);
    return count_ctx(b, &c);
}

/* ======================= generateMoves ======================= */

/* CMove encoding (chess.h:240-243) */
static inline void emit_move(uint16_t **o, int from, int to, int fl)
{
    *(*o)++ = (uint16_t)(((fl & 0xF) << 12) | ((to & 0x3F) << 6) | (from & 0x3F));
}
#define EMIT(from, to, fl) emit_move(&o, (from), (to), (fl))

/* addCompactPawnMoves (MGB.h:1717-1738): promotions in the order N, B, Q, R */
#define EMIT_PAWN(from, dstbb, fl)                                              \
    do {                                                                       \
        int to_ = lsb(dstbb);                                                  \
        if ((dstbb) & (RANK_1 | RANK_8)) {                                     \
            EMIT(from, to_, (fl) | F_PROMO_N);                                 \
            EMIT(from, to_, (fl) | F_PROMO_B);                                 \
            EMIT(from, to_, (fl) | F_PROMO_Q);                                 \
            EMIT(from, to_, (fl) | F_PROMO_R);                                 \
        } else {                                                               \
            EMIT(from, to_, (fl));                                             \
        }                                                                      \
    } while (0)

/* generateMovesOutOfCheck (MGB.h:2266-2463); the host flavour leaves the
 * capture flag off every non-pawn move here. */
static u32 gen_evasions(const or_board *b, const ctx_t *c, uint16_t *out)
{
    uint16_t *o = out;
    int side = c->side;
    for (u64 s = T_KING[c->ksq] & ~(c->threat | c->mine); s; s &= s - 1) EMIT(c->ksq, lsb(s), 0);
    u64 att = checkers(b, c);
    if (att && !several(att)) {
        u64 safe = att | T_BETWEEN[c->ksq][lsb(att)];
        u64 mine = c->mine & ~c->pinned;
        u64 tgt = ep_target(b, side);
        u64 victim = side ? up(tgt) : down(tgt);
        if (victim != att) tgt = 0;
        for (u64 pw = c->pawns & mine; pw; pw &= pw - 1) {
            u64 p = pw & (0 - pw);
            int from = lsb(p);
            u64 d = push1(side, p) & ~c->occ;
            if (d) {
                if (d & safe) {
                    EMIT_PAWN(from, d, 0);
                } else {
                    u64 d2 = push1(side, d & double_rank(side)) & safe & ~c->occ;
                    if (d2) EMIT(from, lsb(d2), F_DOUBLE);
                }
            }
            u64 caps = cap_west(side, p) | cap_east(side, p);
            u64 hit = caps & c->theirs & safe;
            if (hit) EMIT_PAWN(from, hit, F_CAPTURE);
            u64 epd = caps & tgt;
            if (epd) EMIT(from, lsb(epd), F_EP);
        }
        for (u64 s = b->knights & mine; s; s &= s - 1)
            for (u64 m = T_KNIGHT[lsb(s)] & safe; m; m &= m - 1) EMIT(lsb(s), lsb(m), 0);
        for (u64 s = b->bishop_queens & mine; s; s &= s - 1)
            for (u64 m = bishop_one(s & (0 - s), ~c->occ) & safe; m; m &= m - 1) EMIT(lsb(s), lsb(m), 0);
        for (u64 s = b->rook_queens & mine; s; s &= s - 1)
            for (u64 m = rook_one(s & (0 - s), ~c->occ) & safe; m; m &= m - 1) EMIT(lsb(s), lsb(m), 0);
    }
    return (u32)(o - out);
}

/* generateMoves, host flavour (MGB.h:2469-2823): order king, knights,
 * pinned B/Q, B/Q, pinned R/Q, R/Q, en passant, pinned pawns, pawns,
 * castles.  Non-pawn captures carry the capture flag (MGB.h:2525-2529). */
uint32_t or_generate_moves(const or_board *b, uint16_t *out)
{
    ctx_t cc, *c = &cc;
    ctx_init(c, b);
    if (c->threat & c->king) return gen_evasions(b, c, out);
    uint16_t *o = out;
    int side = c->side;
#define CAPF(dstbb) (((dstbb) & c->theirs) ? F_CAPTURE : 0)
    for (u64 s = T_KING[c->ksq] & ~(c->threat | c->mine); s; s &= s - 1)
        EMIT(c->ksq, lsb(s), CAPF(s & (0 - s)));
    for (u64 s = b->knights & c->mine & ~c->pinned; s; s &= s - 1)
        for (u64 m = T_KNIGHT[lsb(s)] & ~c->mine; m; m &= m - 1) EMIT(lsb(s), lsb(m), CAPF(m & (0 - m)));
    u64 my_bq = b->bishop_queens & c->mine, my_rq = b->rook_queens & c->mine;
    for (u64 s = my_bq & c->pinned; s; s &= s - 1)
        for (u64 m = bishop_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]; m; m &= m - 1)
            EMIT(lsb(s), lsb(m), CAPF(m & (0 - m)));
    for (u64 s = my_bq & ~c->pinned; s; s &= s - 1)
        for (u64 m = bishop_one(s & (0 - s), ~c->occ) & ~c->mine; m; m &= m - 1)
            EMIT(lsb(s), lsb(m), CAPF(m & (0 - m)));
    for (u64 s = my_rq & c->pinned; s; s &= s - 1)
        for (u64 m = rook_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]; m; m &= m - 1)
            EMIT(lsb(s), lsb(m), CAPF(m & (0 - m)));
    for (u64 s = my_rq & ~c->pinned; s; s &= s - 1)
        for (u64 m = rook_one(s & (0 - s), ~c->occ) & ~c->mine; m; m &= m - 1)
            EMIT(lsb(s), lsb(m), CAPF(m & (0 - m)));
#undef CAPF
    u64 my_pawns = c->pawns & c->mine;
    u64 tgt = ep_target(b, side);
    if (tgt) {
        u64 victim = side ? up(tgt) : down(tgt);
        for (u64 s = (right1(victim) | left1(victim)) & my_pawns; s; s &= s - 1)
            if (ep_ok(c, s & (0 - s), tgt, victim)) EMIT(lsb(s), lsb(tgt), F_EP);
    }
    for (u64 s = my_pawns & c->pinned; s; s &= s - 1) {
        u64 p = s & (0 - s);
        int from = lsb(p);
        u64 line = T_LINE[from][c->ksq];
        u64 d = push1(side, p) & line & ~c->occ;
        if (d) {
            EMIT(from, lsb(d), 0);
            u64 d2 = push1(side, d & double_rank(side)) & ~c->occ;
            if (d2) EMIT(from, lsb(d2), F_DOUBLE);
        }
        u64 x = (cap_west(side, p) & line) | (cap_east(side, p) & line);
        if (x & c->theirs) EMIT_PAWN(from, x, F_CAPTURE);
    }
    for (u64 s = my_pawns & ~c->pinned; s; s &= s - 1) {
        u64 p = s & (0 - s);
        int from = lsb(p);
        u64 d = push1(side, p) & ~c->occ;
        if (d) {
            EMIT_PAWN(from, d, 0);
            u64 d2 = push1(side, d & double_rank(side)) & ~c->occ;
            if (d2) EMIT_PAWN(from, d2, F_DOUBLE);
        }
        u64 w = cap_west(side, p) & c->theirs;
        if (w) EMIT_PAWN(from, w, F_CAPTURE);
        u64 e = cap_east(side, p) & c->theirs;
        if (e) EMIT_PAWN(from, e, F_CAPTURE);
    }
    if (castle_ks_ok(b, c)) EMIT(side ? 60 : 4, side ? 62 : 6, F_KCASTLE);
    if (castle_qs_ok(b, c)) EMIT(side ? 60 : 4, side ? 58 : 2, F_QCASTLE);
    return (u32)(o - out);
}

/* ======================= generateBoards ======================= */

/* updateCastleFlag (MGB.h:1302-1340): a move by `mover` landing on (or, when
 * called with the other colour, leaving) a rook corner drops that right. */
static void castle_update(or_board *nb, u64 sq, int mover)
{
    if (mover == 0) {
        if (sq & BB(63)) set_bcastle(nb, st_bcastle(nb) & ~1);
        else if (sq & BB(56)) set_bcastle(nb, st_bcastle(nb) & ~2);
    } else {
        if (sq & BB(7)) set_wcastle(nb, st_wcastle(nb) & ~1);
        else if (sq & BB(0)) set_wcastle(nb, st_wcastle(nb) & ~2);
    }
}

static inline u64 new_white(const or_board *b, int side, u64 src, u64 dst)
{
    return side ? (b->white & ~dst) : ((b->white ^ src) | dst);
}

/* addSlidingMove (MGB.h:1342-1397) */
static void bd_slider(or_board **o, const or_board *b, u64 src, u64 dst, int side)
{
    or_board nb;
    nb.bishop_queens = b->bishop_queens & ~dst;
    nb.rook_queens = b->rook_queens & ~dst;
    nb.kings = b->kings & ~dst;
    nb.knights = b->knights & ~dst;
    nb.pawns = b->pawns & ~(dst & INNER_RANKS);
    u64 isb = nb.bishop_queens & src, isr = nb.rook_queens & src;
    nb.bishop_queens ^= isb;
    nb.rook_queens ^= isr;
    if (isb) nb.bishop_queens |= dst;
    if (isr) nb.rook_queens |= dst;
    nb.white = new_white(b, side, src, dst);
    set_side(&nb, !side);
    set_ep(&nb, 0);
    castle_update(&nb, dst, side);
    castle_update(&nb, src, !side);
    *(*o)++ = nb;
}

/* addKnightMove (MGB.h:1400-1438) */
static void bd_knight(or_board **o, const or_board *b, u64 src, u64 dst, int side)
{
    or_board nb;
    nb.bishop_queens = b->bishop_queens & ~dst;
    nb.rook_queens = b->rook_queens & ~dst;
    nb.kings = b->kings & ~dst;
    nb.pawns = b->pawns & ~(dst & INNER_RANKS);
    nb.knights = (b->knights ^ src) | dst;
    nb.white = new_white(b, side, src, dst);
    set_side(&nb, !side);
    set_ep(&nb, 0);
    castle_update(&nb, dst, side);
    *(*o)++ = nb;
}

/* addKingMove (MGB.h:1441-1484) */
static void bd_king(or_board **o, const or_board *b, u64 src, u64 dst, int side)
{
    or_board nb;
    nb.bishop_queens = b->bishop_queens & ~dst;
    nb.rook_queens = b->rook_queens & ~dst;
    nb.knights = b->knights & ~dst;
    nb.pawns = b->pawns & ~(dst & INNER_RANKS);
    nb.kings = (b->kings ^ src) | dst;
    nb.white = new_white(b, side, src, dst);
    if (side) set_bcastle(&nb, 0); else set_wcastle(&nb, 0);
    set_side(&nb, !side);
    set_ep(&nb, 0);
    castle_update(&nb, dst, side);
    *(*o)++ = nb;
}

/* addCastleMove (MGB.h:1487-1522): the rook is toggled, not tested */
static void bd_castle(or_board **o, const or_board *b, int side, int kingside)
{
    int base = side ? 56 : 0;
    u64 kf = BB(base + 4), kt = BB(base + (kingside ? 6 : 2));
    u64 rf = BB(base + (kingside ? 7 : 0)), rt = BB(base + (kingside ? 5 : 3));
    or_board nb;
    nb.bishop_queens = b->bishop_queens;
    nb.pawns = b->pawns;
    nb.knights = b->knights;
    nb.kings = (b->kings ^ kf) | kt;
    nb.rook_queens = (b->rook_queens ^ rf) | rt;
    set_side(&nb, !side);
    set_ep(&nb, 0);
    set_halfmove(&nb, 0);
    if (side == 0) {
        nb.white = (b->white ^ (kf | rf)) | (kt | rt);
        set_wcastle(&nb, 0);
    } else {
        set_bcastle(&nb, 0);
        nb.white = b->white;
    }
    *(*o)++ = nb;
}

/* addSinglePawnMove (MGB.h:1527-1574) */
static void bd_pawn_step(or_board **o, const or_board *b, u64 src, u64 dst, int side, int dbl, int from)
{
    or_board nb;
    nb.bishop_queens = b->bishop_queens & ~dst;
    nb.rook_queens = b->rook_queens & ~dst;
    nb.knights = b->knights & ~dst;
    nb.kings = b->kings;
    nb.pawns = (b->pawns ^ src) | dst;
    nb.white = new_white(b, side, src, dst);
    set_side(&nb, !side);
    set_ep(&nb, dbl ? (from & 7) + 1 : 0);
    set_halfmove(&nb, 0);
    *(*o)++ = nb;
}

/* addEnPassentMove (MGB.h:1576-1618) */
static void bd_ep(or_board **o, const or_board *b, u64 src, u64 dst, int side)
{
    u64 victim = side ? up(dst) : down(dst);
    or_board nb;
    nb.bishop_queens = b->bishop_queens;
    nb.rook_queens = b->rook_queens;
    nb.knights = b->knights;
    nb.kings = b->kings;
    nb.pawns = (b->pawns ^ (victim | src)) | dst;
    nb.white = side ? (b->white ^ victim) : ((b->white ^ src) | dst);
    set_side(&nb, !side);
    set_halfmove(&nb, 0);
    set_ep(&nb, 0);
    *(*o)++ = nb;
}

/* addPawnMoves (MGB.h:1622-1699): promotions N, B, Q, R */
static void bd_pawn(or_board **o, const or_board *b, u64 src, u64 dst, int side)
{
    if (!(dst & (RANK_1 | RANK_8))) {
        bd_pawn_step(o, b, src, dst, side, 0, 0);
        return;
    }
    or_board nb;
    nb.kings = b->kings;
    nb.white = new_white(b, side, src, dst);
    nb.pawns = b->pawns ^ src;
    set_side(&nb, !side);
    set_ep(&nb, 0);
    set_halfmove(&nb, 0);
    castle_update(&nb, dst, side);
    nb.knights = b->knights | dst;
    nb.bishop_queens = b->bishop_queens & ~dst;
    nb.rook_queens = b->rook_queens & ~dst;
    *(*o)++ = nb;
    nb.knights = b->knights & ~dst;
    nb.bishop_queens = b->bishop_queens | dst;
    nb.rook_queens = b->rook_queens & ~dst;
    *(*o)++ = nb;
    nb.rook_queens = b->rook_queens | dst;
    *(*o)++ = nb;
    nb.bishop_queens = b->bishop_queens & ~dst;
    *(*o)++ = nb;
}

/* generateBoardsOutOfCheck (MGB.h:1741-1933) */
static u32 boards_evasions(const or_board *b, const ctx_t *c, or_board *out)
{
    or_board *o = out;
    int side = c->side;
    for (u64 s = T_KING[c->ksq] & ~(c->threat | c->mine); s; s &= s - 1)
        bd_king(&o, b, c->king, s & (0 - s), side);
    u64 att = checkers(b, c);
    if (att && !several(att)) {
        u64 safe = att | T_BETWEEN[c->ksq][lsb(att)];
        u64 mine = c->mine & ~c->pinned;
        u64 tgt = ep_target(b, side);
        u64 victim = side ? up(tgt) : down(tgt);
        if (victim != att) tgt = 0;
        for (u64 pw = c->pawns & mine; pw; pw &= pw - 1) {
            u64 p = pw & (0 - pw);
            u64 d = push1(side, p) & ~c->occ;
            if (d) {
                if (d & safe) {
                    bd_pawn(&o, b, p, d, side);
                } else {
                    u64 d2 = push1(side, d & double_rank(side)) & safe & ~c->occ;
                    if (d2) bd_pawn_step(&o, b, p, d2, side, 1, lsb(p));
                }
            }
            u64 caps = cap_west(side, p) | cap_east(side, p);
            u64 hit = caps & c->theirs & safe;
            if (hit) bd_pawn(&o, b, p, hit, side);
            u64 epd = caps & tgt;
            if (epd) bd_ep(&o, b, p, epd, side);
        }
        for (u64 s = b->knights & mine; s; s &= s - 1)
            for (u64 m = T_KNIGHT[lsb(s)] & safe; m; m &= m - 1) bd_knight(&o, b, s & (0 - s), m & (0 - m), side);
        for (u64 s = b->bishop_queens & mine; s; s &= s - 1)
            for (u64 m = bishop_one(s & (0 - s), ~c->occ) & safe; m; m &= m - 1)
                bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
        for (u64 s = b->rook_queens & mine; s; s &= s - 1)
            for (u64 m = rook_one(s & (0 - s), ~c->occ) & safe; m; m &= m - 1)
                bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
    }
    return (u32)(o - out);
}

/* generateBoards (MGB.h:1940-2261): order en passant, pinned pawns, pawns,
 * castles, king, knights, pinned B/Q, B/Q, pinned R/Q, R/Q. */
uint32_t or_generate_boards(const or_board *b, or_board *out)
{
    ctx_t cc, *c = &cc;
    ctx_init(c, b);
    if (c->threat & c->king) return boards_evasions(b, c, out);
    or_board *o = out;
    int side = c->side;
    u64 my_pawns = c->pawns & c->mine;
    u64 tgt = ep_target(b, side);
    if (tgt) {
        u64 victim = side ? up(tgt) : down(tgt);
        for (u64 s = (right1(victim) | left1(victim)) & my_pawns; s; s &= s - 1)
            if (ep_ok(c, s & (0 - s), tgt, victim)) bd_ep(&o, b, s & (0 - s), tgt, side);
    }
    for (u64 s = my_pawns & c->pinned; s; s &= s - 1) {
        u64 p = s & (0 - s);
        int from = lsb(p);
        u64 line = T_LINE[from][c->ksq];
        u64 d = push1(side, p) & line & ~c->occ;
        if (d) {
            bd_pawn_step(&o, b, p, d, side, 0, from);
            u64 d2 = push1(side, d & double_rank(side)) & ~c->occ;
            if (d2) bd_pawn_step(&o, b, p, d2, side, 1, from);
        }
        u64 x = (cap_west(side, p) & line) | (cap_east(side, p) & line);
        if (x & c->theirs) bd_pawn(&o, b, p, x, side);
    }
    for (u64 s = my_pawns & ~c->pinned; s; s &= s - 1) {
        u64 p = s & (0 - s);
        u64 d = push1(side, p) & ~c->occ;
        if (d) {
            bd_pawn(&o, b, p, d, side);
            u64 d2 = push1(side, d & double_rank(side)) & ~c->occ;
            if (d2) bd_pawn_step(&o, b, p, d2, side, 1, lsb(p));
        }
        u64 w = cap_west(side, p) & c->theirs;
        if (w) bd_pawn(&o, b, p, w, side);
        u64 e = cap_east(side, p) & c->theirs;
        if (e) bd_pawn(&o, b, p, e, side);
    }
    if (castle_ks_ok(b, c)) bd_castle(&o, b, side, 1);
    if (castle_qs_ok(b, c)) bd_castle(&o, b, side, 0);
    for (u64 s = T_KING[c->ksq] & ~(c->threat | c->mine); s; s &= s - 1)
        bd_king(&o, b, c->king, s & (0 - s), side);
    for (u64 s = b->knights & c->mine & ~c->pinned; s; s &= s - 1)
        for (u64 m = T_KNIGHT[lsb(s)] & ~c->mine; m; m &= m - 1) bd_knight(&o, b, s & (0 - s), m & (0 - m), side);
    u64 my_bq = b->bishop_queens & c->mine, my_rq = b->rook_queens & c->mine;
    for (u64 s = my_bq & c->pinned; s; s &= s - 1)
        for (u64 m = bishop_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]; m; m &= m - 1)
            bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
    for (u64 s = my_bq & ~c->pinned; s; s &= s - 1)
        for (u64 m = bishop_one(s & (0 - s), ~c->occ) & ~c->mine; m; m &= m - 1)
            bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
    for (u64 s = my_rq & c->pinned; s; s &= s - 1)
        for (u64 m = rook_one(s & (0 - s), ~c->occ) & ~c->mine & T_LINE[lsb(s)][c->ksq]; m; m &= m - 1)
            bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
    for (u64 s = my_rq & ~c->pinned; s; s &= s - 1)
        for (u64 m = rook_one(s & (0 - s), ~c->occ) & ~c->mine; m; m &= m - 1)
            bd_slider(&o, b, s & (0 - s), m & (0 - m), side);
    return (u32)(o - out);
}

/* ======================= makeMove ======================= */

/* makeMove<c, false> (MGB.h:3310-3570) with EXACT_EN_PASSENT_FLAGGING. */
void or_make_move(or_board *b, uint16_t mv)
{
    int from = mv & 63, to = (mv >> 6) & 63, fl = (mv >> 12) & 15;
    int side = st_side(b);
    u64 src = BB(from), dst = BB(to);
    u64 queens = b->bishop_queens & b->rook_queens;
    enum { P = 1, N, B, R, Q, K } piece;
    if (b->kings & src) piece = K;
    else if (b->knights & src) piece = N;
    else if (b->pawns & INNER_RANKS & src) piece = P;
    else if (queens & src) piece = Q;
    else if (b->bishop_queens & src) piece = B;
    else piece = R;
    if (fl == 8 || fl == 12) piece = N;
    else if (fl == 9 || fl == 13) piece = B;
    else if (fl == 10 || fl == 14) piece = R;
    else if (fl == 11 || fl == 15) piece = Q;

    u64 clear = ~(src | dst);
    b->bishop_queens &= clear;
    b->rook_queens &= clear;
    b->kings &= clear;
    b->knights &= clear;
    b->pawns &= ~((src | dst) & INNER_RANKS);
    if (piece == K) {
        b->kings |= dst;
        if (side) set_bcastle(b, 0); else set_wcastle(b, 0);
    }
    if (piece == N) b->knights |= dst;
    if (piece == P) b->pawns |= dst;
    if (piece == B || piece == Q) b->bishop_queens |= dst;
    if (piece == R || piece == Q) b->rook_queens |= dst;
    b->white = side ? (b->white & ~dst) : ((b->white ^ src) | dst);

    if (fl == F_EP) {
        u64 victim = side ? up(dst) : down(dst);
        b->pawns &= ~(victim & INNER_RANKS);
        if (side) b->white &= ~victim;
    }
    if (fl == F_KCASTLE || fl == F_QCASTLE) {
        int base = side ? 56 : 0;
        u64 rf = BB(base + (fl == F_KCASTLE ? 7 : 0)), rt = BB(base + (fl == F_KCASTLE ? 5 : 3));
        b->rook_queens = (b->rook_queens ^ rf) | rt;
        if (!side) b->white = (b->white ^ rf) | rt;
    }
    set_side(b, !side);
    set_ep(b, 0);
    castle_update(b, dst, side);
    if (piece == R) castle_update(b, src, !side);
    if (fl == F_DOUBLE) {
        u64 pawns = b->pawns & INNER_RANKS;
        u64 occ = b->kings | pawns | b->knights | b->bishop_queens | b->rook_queens;
        u64 enemy = side ? b->white : (occ & ~b->white);
        if ((right1(dst) | left1(dst)) & pawns & enemy) set_ep(b, (from & 7) + 1);
    }
}

/* ======================= perft ======================= */

uint64_t or_perft(const or_board *b, int depth)
{
    if (depth <= 0) return 1;
    if (depth == 1) return or_count_moves(b);
    or_board kids[256];
    u32 n = or_generate_boards(b, kids);
    uint64_t sum = 0;
    for (u32 i = 0; i < n; i++) sum += or_perft(&kids[i], depth - 1);
    return sum;
}

uint64_t or_perft_moves(const or_board *b, int depth)
{
    if (depth <= 0) return 1;
    if (depth == 1) return or_count_moves(b);
    uint16_t mv[256];
    u32 n = or_generate_moves(b, mv);
    uint64_t sum = 0;
    for (u32 i = 0; i < n; i++) {
        or_board k = *b;
        or_make_move(&k, mv[i]);
        sum += or_perft_moves(&k, depth - 1);
    }
    return sum;
}

uint32_t or_perft_divide(const or_board *b, int depth, uint16_t *moves, uint64_t *counts)
{
    u32 n = or_generate_moves(b, moves);
    for (u32 i = 0; i < n; i++) {
        or_board k = *b;
        or_make_move(&k, moves[i]);
        counts[i] = or_perft(&k, depth - 1);
    }
    return n;
}

typedef struct {
    const or_board *b;
    const uint8_t *d;
    uint64_t *out;
    u32 n;
    volatile u32 next;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *j = (batch_job *)arg;
    for (;;) {
        u32 i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (i >= j->n) break;
        j->out[i] = or_perft(&j->b[i], j->d[i]);
    }
    return NULL;
}

double or_perft_batch(const or_board *b, const uint8_t *depths, uint32_t n, uint64_t *out, int nthreads)
{
    struct timespec t0, t1;
    batch_job job = {b, depths, out, n, 0};
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 512) nthreads = 512;
    pthread_t th[512];
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &job);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ======================= inputs ======================= */

void or_start_position(or_board *out)
{
    or_board_from_fen("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1", out);
}

/* readFENString (util.cpp:189-280) then board088ToHexBB (util.cpp:92-140):
 * board, side, castling letters, en-passant file; the half-move and
 * full-move counters are not read (half-move stays 0). */
int or_board_from_fen(const char *fen, or_board *out)
{
    memset(out, 0, sizeof(*out));
    int row = 0, col = 0, i = 0;
    for (; fen[i]; i++) {
        char ch = fen[i];
        if (ch == '/' || ch == '\\') {
            row++;
            col = 0;
        } else if (ch >= '1' && ch <= '8') {
            col += ch - '0';
        } else {
            const char *pieces = "PNBRQKpnbrqk";
            const char *hit = strchr(pieces, ch);
            if (hit && ch) {
                int k = (int)(hit - pieces);
                int sq = (7 - row) * 8 + col;
                if (row <= 7 && col <= 7) {
                    u64 bit = BB(sq);
                    int kind = k % 6;
                    if (k < 6) out->white |= bit;
                    if (kind == 0) out->pawns |= bit;
                    if (kind == 1) out->knights |= bit;
                    if (kind == 2 || kind == 4) out->bishop_queens |= bit;
                    if (kind == 3 || kind == 4) out->rook_queens |= bit;
                    if (kind == 5) out->kings |= bit;
                }
                col++;
            }
        }
        if (row >= 7 && col == 8) break;
    }
    if (!fen[i]) return -1;
    i++;
    while (fen[i] == ' ') i++;
    int side = (fen[i] == 'b' || fen[i] == 'B') ? 1 : 0;
    if (fen[i]) i++;
    while (fen[i] == ' ') i++;
    int wc = 0, bc = 0;
    while (fen[i] && fen[i] != ' ') {
        if (fen[i] == 'k') bc |= 1;
        if (fen[i] == 'q') bc |= 2;
        if (fen[i] == 'K') wc |= 1;
        if (fen[i] == 'Q') wc |= 2;
        i++;
    }
    while (fen[i] == ' ') i++;
    int ep = (fen[i] >= 'a' && fen[i] <= 'h') ? fen[i] - 'a' + 1 : 0;
    /* pawns on ranks 1 and 8 would collide with the packed state; the
     * reference's board088ToHexBB ORs them in before writing the state
     * fields, so the state fields win on those bits */
    out->pawns &= INNER_RANKS;
    set_wcastle(out, wc);
    set_bcastle(out, bc);
    set_ep(out, ep);
    set_halfmove(out, 0);
    set_side(out, side);
    return 0;
}

/* ======================= seeded playouts ======================= */

static inline u64 sm_next(u64 *s)
{
    u64 z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void or_playouts(uint64_t seed, uint32_t n, int min_plies, int max_plies, int min_moves,
                 int depth_lo, int depth_hi, or_board *out, uint8_t *depths)
{
    or_board start;
    or_start_position(&start);
    if (min_moves < 1) min_moves = 1;
    for (u32 i = 0; i < n; i++) {
        for (u64 a = 0;; a++) {
            u64 s = seed ^ ((u64)i << 32) ^ (a * 0xA24BAED4963EE407ull);
            int plies = min_plies + (int)(sm_next(&s) % (u64)(max_plies - min_plies + 1));
            or_board p = start;
            int ok = 1;
            for (int k = 0; k < plies; k++) {
                uint16_t mv[256];
                u32 m = or_generate_moves(&p, mv);
                if (!m) { ok = 0; break; }
                or_make_move(&p, mv[sm_next(&s) % m]);
            }
            if (ok && (int)or_count_moves(&p) >= min_moves) {
                out[i] = p;
                break;
            }
        }
        if (depths) {
            u64 s = seed ^ ((u64)i << 32) ^ 0x5851F42D4C957F2Dull;
            depths[i] = (uint8_t)(depth_lo + (int)(sm_next(&s) % (u64)(depth_hi - depth_lo + 1)));
        }
    }
}

uint64_t or_board_hash(const or_board *b)
{
    const u64 *w = (const u64 *)b;
    u64 h = 0x84222325CBF29CE4ull;
    for (int i = 0; i < 6; i++) {
        h ^= w[i];
        h *= 0x100000001B3ull;
        h ^= h >> 29;
    }
    return h;
}
