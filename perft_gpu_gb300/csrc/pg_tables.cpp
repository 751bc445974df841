// pg_tables.cpp -- host construction of the lookup tables: knight patterns
// and fancy magic bitboards found by our own seeded search (the attack sets
// equal the reference's tables, MoveGeneratorBitboard.h:1024-1076 and
// Magics.cpp:231-339; the magic factors and layout are our own).  The same
// tables feed the byte-lookup variant: per square, each distinct attack set
// gets a byte id in enumeration order, and the byte table maps the magic
// index to that id.
#include <vector>

#include "pg_tables.h"

namespace pg {

static u64 host_rays(int sq, u64 occ, bool rook)
{
    static const int rd[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
    static const int bd[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
    const int(*d)[2] = rook ? rd : bd;
    u64 att = 0;
    for (int k = 0; k < 4; k++) {
        int r = sq >> 3, f = sq & 7;
        for (;;) {
            r += d[k][0];
            f += d[k][1];
            if (r < 0 || r > 7 || f < 0 || f > 7) break;
            att |= 1ull << (r * 8 + f);
            if (occ & (1ull << (r * 8 + f))) break;
        }
    }
    return att;
}

static int build_square(MagicSq& e, int sq, bool rook, u32& offset, u32& uniq, HostTables& t, u64& rng)
{
    const u64 RANK1 = 0xFFull, RANK8 = 0xFF00000000000000ull, FA = 0x0101010101010101ull, FH = FA << 7;
    const u64 edges = ((RANK1 | RANK8) & ~(RANK1 << (8 * (sq >> 3)))) | ((FA | FH) & ~(FA << (sq & 7)));
    const u64 mask = host_rays(sq, 0, rook) & ~edges;
    const int bits = __builtin_popcountll(mask);
    const int size = 1 << bits;
    std::vector<u64> occ(size), att(size);
    std::vector<int> epoch(size, -1);
    std::vector<u64> slot(size);
    int n = 0;
    u64 sub = 0;
    do {
        occ[n] = sub;
        att[n] = host_rays(sq, sub, rook);
        n++;
        sub = (sub - mask) & mask;
    } while (sub);
    auto next = [&]() {
        rng ^= rng >> 12;
        rng ^= rng << 25;
        rng ^= rng >> 27;
        return rng * 0x2545F4914F6CDD1Dull;
    };
    const int shift = 64 - bits;
    u64 magic = 0;
    for (int attempt = 0; attempt < 100000000; attempt++) {
        const u64 m = next() & next() & next();
        if (__builtin_popcountll((mask * m) & 0xFF00000000000000ull) < 6) continue;
        bool ok = true;
        for (int i = 0; i < n && ok; i++) {
            const int idx = (int)((occ[i] * m) >> shift);
            if (epoch[idx] != attempt) {
                epoch[idx] = attempt;
                slot[idx] = att[i];
            } else if (slot[idx] != att[i]) {
                ok = false;
            }
        }
        if (ok) {
            magic = m;
            break;
        }
    }
    if (!magic) return -1;
    // unique attack sets of this square, numbered in enumeration order
    std::vector<u64> uniq_sets;
    for (int i = 0; i < n; i++) {
        const int idx = (int)((occ[i] * magic) >> shift);
        t.attacks[offset + idx] = att[i];
        int id = -1;
        for (size_t u = 0; u < uniq_sets.size(); u++)
            if (uniq_sets[u] == att[i]) {
                id = (int)u;
                break;
            }
        if (id < 0) {
            id = (int)uniq_sets.size();
            uniq_sets.push_back(att[i]);
        }
        if (id > 255) return -2;
        t.bytes[offset + idx] = (unsigned char)id;
    }
    e.mask = mask;
    e.magic = magic;
    e.offset = offset;
    e.shift = (u32)shift;
    e.uniq = uniq;
    e.pad = 0;
    for (size_t u = 0; u < uniq_sets.size(); u++) t.unique[uniq + u] = uniq_sets[u];
    offset += (u32)size;
    uniq += (u32)uniq_sets.size();
    return 0;
}

int build_tables(HostTables& t)
{
    t.attacks.assign(MAGIC_TABLE_ENTRIES, 0);
    t.bytes.assign(MAGIC_TABLE_ENTRIES, 0);
    t.unique.assign(UNIQUE_TOTAL, 0);
    u32 offset = 0, uniq = 0;
    u64 rng = 0x2545F4914F6CDD1Dull;
    for (int s = 0; s < 64; s++)
        if (build_square(t.rook[s], s, true, offset, uniq, t, rng)) return -1;
    if (uniq != (u32)UNIQUE_ROOK) return -2;
    for (int s = 0; s < 64; s++)
        if (build_square(t.bishop[s], s, false, offset, uniq, t, rng)) return -1;
    if (offset != (u32)MAGIC_TABLE_ENTRIES || uniq != (u32)UNIQUE_TOTAL) return -3;
    for (int s = 0; s < 64; s++) {
        const u64 b = 1ull << s;
        const u64 a = ((b >> 1) & ~(0x0101010101010101ull << 7)) | ((b << 1) & ~0x0101010101010101ull);
        const u64 c = ((b >> 2) & 0x3F3F3F3F3F3F3F3Full) | ((b << 2) & 0xFCFCFCFCFCFCFCFCull);
        t.knight[s] = (a << 16) | (a >> 16) | (c << 8) | (c >> 8);
        const u64 row = b | a;
        t.king[s] = ((b >> 1) & ~(0x0101010101010101ull << 7)) | ((b << 1) & ~0x0101010101010101ull) | (row << 8) |
                    (row >> 8);
        const int d = (s >> 3) - (s & 7);
        t.diag[s] = d >= 0 ? (0x8040201008040201ull << (8 * d)) : (0x8040201008040201ull >> (-8 * d));
        const u64 not_a = ~0x0101010101010101ull, not_h = ~0x8080808080808080ull;
        t.pawn_checks[0][s] = ((b << 9) & not_a) | ((b << 7) & not_h);  // black pawns above a white king
        t.pawn_checks[1][s] = ((b >> 7) & not_a) | ((b >> 9) & not_h);  // white pawns below a black king
    }
    return 0;
}


const HostTables* host_tables()
{
    static HostTables* t = nullptr;
    static int status = 1;
    if (status == 1) {
        t = new HostTables();
        status = build_tables(*t);
    }
    return status == 0 ? t : nullptr;
}

}  // namespace pg
