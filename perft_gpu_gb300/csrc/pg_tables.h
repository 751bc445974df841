// pg_tables.h -- host copy of the move generator's lookup tables.
#pragma once
#include <vector>

#include "pg_types.h"

namespace pg {

struct MagicSq {
    u64 mask;
    u64 magic;
    u32 offset;  // first entry of this square in the attack / byte table
    u32 shift;   // 64 - relevant occupancy bits
    u32 uniq;    // byte-lookup: first unique attack set of this square
    u32 pad;
};
constexpr int MAGIC_TABLE_ENTRIES = 102400 + 5248;  // rook + bishop, variable shift
constexpr int UNIQUE_ROOK = 4900;                   // distinct rook attack sets over all squares
constexpr int UNIQUE_BISHOP = 1428;
constexpr int UNIQUE_TOTAL = UNIQUE_ROOK + UNIQUE_BISHOP;

struct HostTables {
    MagicSq rook[64], bishop[64];
    std::vector<u64> attacks;
    std::vector<unsigned char> bytes;
    std::vector<u64> unique;
    u64 knight[64];
    u64 king[64];
    u64 diag[64];  // the a1-h8 diagonal through each square
    u64 pawn_checks[2][64];  // squares from which an enemy pawn attacks a king of side s on square q
};

// built once per process; nullptr if the search failed
const HostTables* host_tables();

}  // namespace pg
