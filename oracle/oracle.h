/*
 * oracle.h -- CPU restatement of the reference perft move generator.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the GPU engine's
 * counts are compared against.  It is loaded by tests/, by __graft_entry__.smoke() and
 * by bench.py's CPU-baseline / reference leg, and by nothing else.  The product
 * (perft_gpu_gb300/) never links, loads or calls it.
 *
 * Every function restates the algorithm of the reference (sarona-RD/perft_gpu)
 * at the file:line given beside it; the 48-byte board layout and the 16-bit
 * move encoding are the reference's own (chess.h:207-230, chess.h:234-293).
 * Parity of this restatement is pinned against the reference itself, compiled
 * from its sources by oracle/build_ref.sh into oracle/_ref/, and against the
 * golden vectors in tests/golden/ that the reference produced.
 */
#ifndef PERFT_ORACLE_H
#define PERFT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same bytes as HexaBitBoardPosition (chess.h:207-230). */
typedef struct or_board {
    uint64_t white;          /* whitePieces                                  */
    uint64_t pawns;          /* pawns on ranks 2-7 + packed game state       */
    uint64_t knights;
    uint64_t bishop_queens;
    uint64_t rook_queens;
    uint64_t kings;
} or_board;

/* Slider attack method: 0 = Kogge-Stone fills (USE_SLIDING_LUT 0),
 * 1 = fancy magic lookup (the reference's default build).  Counts are the
 * same either way; only the speed differs. */
void     or_init(int slider_mode);

/* Utils::readFENString + board088ToHexBB (util.cpp:189-280, util.cpp:92-140). */
int      or_board_from_fen(const char *fen, or_board *out);

/* MoveGeneratorBitboard::countMoves<c> (MoveGeneratorBitboard.h:3008-3295,
 * out of check 2825-3002). */
uint32_t or_count_moves(const or_board *b);

/* generateMoves<c>, host flavour (MoveGeneratorBitboard.h:2469-2823,
 * out of check 2266-2463).  moves must hold 256 entries. */
uint32_t or_generate_moves(const or_board *b, uint16_t *moves);

/* generateBoards<c> (MoveGeneratorBitboard.h:1940-2261, out of check
 * 1741-1933, helpers 1302-1738).  out must hold 256 boards. */
uint32_t or_generate_boards(const or_board *b, or_board *out);

/* makeMove<c,false> with exact en-passant flagging
 * (MoveGeneratorBitboard.h:3310-3570). */
void     or_make_move(or_board *b, uint16_t move);

/* perft_bb (perft_bb.h:79-101): generateBoards recursion, countMoves leaf. */
uint64_t or_perft(const or_board *b, int depth);

/* The same count through generateMoves + makeMove (the primitives of the
 * reference's GPU BFS, perft_bb.h:601-1138). */
uint64_t or_perft_moves(const or_board *b, int depth);

/* Divided perft in generateMoves order: moves[i] and counts[i] for every
 * legal root move; returns the number of root moves. depth >= 1. */
uint32_t or_perft_divide(const or_board *b, int depth, uint16_t *moves,
                         uint64_t *counts);

/* perft of n positions over nthreads POSIX threads (dynamic assignment);
 * depths[i] in 0..15.  Returns wall seconds. */
double   or_perft_batch(const or_board *b, const uint8_t *depths, uint32_t n,
                        uint64_t *out, int nthreads);

/* Seeded random legal playouts from the initial position.  Position i is
 * the first accepted attempt a = 0, 1, ... of: plies = min_plies +
 * r() % (max_plies - min_plies + 1), then per ply pick generateMoves[r() % n]
 * and makeMove; accepted when every ply had a move and the final position
 * has at least min_moves legal moves.  r() is splitmix64 over the state
 * seed_state(seed, i, a).  depth_lo/depth_hi: depths[i] = depth_lo +
 * r() % (depth_hi - depth_lo + 1) from a separate stream (may be NULL). */
void     or_playouts(uint64_t seed, uint32_t n, int min_plies, int max_plies,
                     int min_moves, int depth_lo, int depth_hi,
                     or_board *out, uint8_t *depths);

/* The initial position. */
void     or_start_position(or_board *out);

/* Stable 64-bit fingerprint of a board (for fixtures). */
uint64_t or_board_hash(const or_board *b);

#ifdef __cplusplus
}
#endif
#endif
