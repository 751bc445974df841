// pg_host.cpp -- host-only parts of the C ABI: FEN input.
#include <cstring>

#include "../../include/perft_gb300.h"

extern "C" int pg_board_from_fen(const char* fen, pg_board* out)
{
    // Utils::readFENString (util.cpp:189-280) followed by board088ToHexBB
    // (util.cpp:92-140): piece placement, side, castling letters, en-passant
    // file; the half-move and full-move counters are not read, so the
    // half-move field is 0.  Pawns on ranks 1 and 8 lose the bits the
    // packed state occupies, as in the reference.
    if (!fen || !out) return PG_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    int row = 0, col = 0, i = 0;
    bool done = false;
    for (; fen[i]; i++) {
        const char ch = fen[i];
        if (ch == '/' || ch == '\\') {
            row++;
            col = 0;
        } else if (ch >= '1' && ch <= '8') {
            col += ch - '0';
        } else {
            static const char pieces[] = "PNBRQKpnbrqk";
            const char* hit = strchr(pieces, ch);
            if (hit) {
                const int k = (int)(hit - pieces), kind = k % 6;
                if (row <= 7 && col <= 7) {
                    const uint64_t bit = 1ull << ((7 - row) * 8 + col);
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
        if (row >= 7 && col == 8) {
            done = true;
            break;
        }
    }
    if (!done) return PG_ERR_INVALID_ARGUMENT;
    i++;
    while (fen[i] == ' ') i++;
    const int side = (fen[i] == 'b' || fen[i] == 'B') ? 1 : 0;
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
    const int ep = (fen[i] >= 'a' && fen[i] <= 'h') ? fen[i] - 'a' + 1 : 0;
    out->pawns &= 0x00FFFFFFFFFFFF00ull;
    out->pawns |= (uint64_t)wc | ((uint64_t)bc << 2) | ((uint64_t)ep << 4) | ((uint64_t)side << 63);
    return PG_OK;
}
