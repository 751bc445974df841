// ref_shim.cpp -- extern "C" entry points over the reference's own host move
// generator, compiled unchanged from its sources by oracle/build_ref.sh.
//
// TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement (oracle.c) and
// to generate the golden vectors in tests/golden/.  Nothing in the product
// loads it.  The reference's perft_bb recursion lives in a CUDA-only header
// (perft_bb.h:79-101), so ref_perft below calls the same two primitives
// (generateBoards, countMoves) in the same recursion.
#define SKIP_CUDA_CODE
#include "chess.h"
#include "MoveGeneratorBitboard.h"

#include <atomic>
#include <chrono>
#include <cstdint>
#include <thread>
#include <vector>

static uint32 ref_count(HexaBitBoardPosition *p)
{
    return p->chance == BLACK ? MoveGeneratorBitboard::countMoves<BLACK>(p)
                              : MoveGeneratorBitboard::countMoves<WHITE>(p);
}

static uint32 ref_boards(HexaBitBoardPosition *p, HexaBitBoardPosition *c)
{
    return p->chance == BLACK ? MoveGeneratorBitboard::generateBoards<BLACK>(p, c)
                              : MoveGeneratorBitboard::generateBoards<WHITE>(p, c);
}

static uint64 ref_perft_rec(HexaBitBoardPosition *p, int d)
{
    if (d <= 0) return 1;
    if (d == 1) return ref_count(p);
    HexaBitBoardPosition kids[MAX_MOVES];
    uint32 n = ref_boards(p, kids);
    uint64 s = 0;
    for (uint32 i = 0; i < n; i++) s += ref_perft_rec(&kids[i], d - 1);
    return s;
}

extern "C" {

void ref_init(void) { MoveGeneratorBitboard::init(); }

int ref_board_from_fen(const char *fen, HexaBitBoardPosition *out)
{
    BoardPosition b;
    char buf[1024];
    strncpy(buf, fen, sizeof(buf) - 1);
    buf[sizeof(buf) - 1] = 0;
    Utils::readFENString(buf, &b);
    Utils::board088ToHexBB(out, &b);
    return 0;
}

uint32_t ref_count_moves(const HexaBitBoardPosition *p)
{
    HexaBitBoardPosition c = *p;
    return ref_count(&c);
}

uint32_t ref_generate_moves(const HexaBitBoardPosition *p, uint16_t *out)
{
    HexaBitBoardPosition c = *p;
    CMove mv[MAX_MOVES];
    uint32 n = c.chance == BLACK ? MoveGeneratorBitboard::generateMoves<BLACK>(&c, mv)
                                 : MoveGeneratorBitboard::generateMoves<WHITE>(&c, mv);
    memcpy(out, mv, n * sizeof(uint16_t));
    return n;
}

uint32_t ref_generate_boards(const HexaBitBoardPosition *p, HexaBitBoardPosition *out)
{
    HexaBitBoardPosition c = *p;
    return ref_boards(&c, out);
}

void ref_make_move(HexaBitBoardPosition *p, uint16_t move)
{
    CMove m;
    memcpy(&m, &move, sizeof(m));
    uint64 h = 0;
    if (p->chance == BLACK)
        MoveGeneratorBitboard::makeMove<BLACK, false>(p, h, m);
    else
        MoveGeneratorBitboard::makeMove<WHITE, false>(p, h, m);
}

uint64_t ref_perft(const HexaBitBoardPosition *p, int depth)
{
    HexaBitBoardPosition c = *p;
    return ref_perft_rec(&c, depth);
}

double ref_perft_batch(const HexaBitBoardPosition *b, const uint8_t *depths, uint32_t n,
                       uint64_t *out, int nthreads)
{
    std::atomic<uint32_t> next(0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    if (nthreads < 1) nthreads = 1;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&] {
            uint32_t i;
            while ((i = next++) < n) {
                HexaBitBoardPosition c = b[i];
                out[i] = ref_perft_rec(&c, depths[i]);
            }
        });
    for (auto &x : th) x.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // extern "C"
