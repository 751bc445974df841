// pg_cli.cpp -- perft_gpu: the command line of the reference's binary
// (perft.cu:14-164) over the C ABI.
//
//   perft_gpu [<fen> [<depth> [<numGPUs> [<launchDepth>]]]] [-divide] [-tt]
//   perft_gpu -records <file> [<depth>] [-tt]
//   ... [-ttload <snapshot>] [-ttsave <snapshot>]   (imply -tt) [-ttmib <MiB>]
//
// Like perft.cu it prints one "GPU Perft" line (launcher.h:1488-1498) per
// depth from 3 to <depth>; depths of 9 and more go through the divided path
// with the host-side complete TT (perft_bb_cpu_launcher, launcher.h:1181-1389)
// and print the per-move lines and the "Perft(NN)" total of dividedPerft
// (launcher.h:1344-1351, 1439).  <numGPUs> other than 1 is reported and one
// GPU is used; <launchDepth> is accepted and ignored (the engine plans its
// own split from the HBM budget).  Records mode follows processPerftRecords
// (launcher.h:1579-1694): each input line is a FEN followed by an occurrence
// count; "<line> <perft> <perft x count>" is appended to <file>.op, and lines
// already present there are skipped, so an interrupted run resumes.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "perft_gb300.h"

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static std::string move_string(pg_move m)
{
    // Utils::getCompactMoveString (utils.h:251-278)
    const int from = m & 63, to = (m >> 6) & 63, cap = (m >> 12) & 4;
    char buf[16];
    snprintf(buf, sizeof(buf), "%c%d%c%c%d ", 'a' + (from & 7), (from >> 3) + 1, cap ? '*' : '-', 'a' + (to & 7),
             (to >> 3) + 1);
    return buf;
}

static uint64_t g_tt_bytes = 0;  // -ttmib: TT size (0 = from the engine's budget)

static int fail(const char* what)
{
    fprintf(stderr, "%s failed: %s\n", what, pg_last_error());
    return 1;
}

static int records_mode(const char* file, int depth, bool tt)
{
    std::string opname = std::string(file) + ".op";
    FILE* in = fopen(file, "rb");
    if (!in) {
        fprintf(stderr, "cannot open %s\n", file);
        return 1;
    }
    size_t done = 0;
    if (FILE* op = fopen(opname.c_str(), "rb")) {
        char line[2048];
        while (fgets(line, sizeof(line), op)) done++;
        fclose(op);
    }
    FILE* op = fopen(opname.c_str(), "ab");
    if (!op) {
        fprintf(stderr, "cannot open %s\n", opname.c_str());
        return 1;
    }
    printf("filename of op: %s\n", opname.c_str());
    std::vector<std::string> lines;
    char line[2048];
    size_t idx = 0;
    while (fgets(line, sizeof(line), in)) {
        if (idx++ < done) continue;  // already processed
        std::string s(line);
        while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
        if (!s.empty()) lines.push_back(s);
    }
    fclose(in);
    const double t0 = now_s();
    pg_opts o{};
    o.use_tt = tt ? 1 : 0;
    o.tt_bytes = g_tt_bytes;
    const size_t B = 4096;
    for (size_t b0 = 0; b0 < lines.size(); b0 += B) {
        const size_t nb = std::min(B, lines.size() - b0);
        std::vector<pg_board> boards(nb);
        std::vector<uint8_t> depths(nb, (uint8_t)depth);
        std::vector<uint64_t> res(nb);
        for (size_t i = 0; i < nb; i++)
            if (pg_board_from_fen(lines[b0 + i].c_str(), &boards[i]) != PG_OK) return fail("FEN");
        if (pg_perft_batch(boards.data(), depths.data(), (uint32_t)nb, res.data(), &o) != PG_OK)
            return fail("pg_perft_batch");
        for (size_t i = 0; i < nb; i++) {
            const std::string& s = lines[b0 + i];
            const size_t sp = s.find_last_of(' ');
            const long long occ = sp == std::string::npos ? 1 : atoll(s.c_str() + sp + 1);
            printf("\n%s\nGPU Perft %d: %llu", s.c_str(), depth, (unsigned long long)res[i]);
            fprintf(op, "%s %llu %llu\n", s.c_str(), (unsigned long long)res[i],
                    (unsigned long long)(res[i] * (unsigned long long)occ));
        }
        fflush(op);
        const double t = now_s() - t0;
        printf("\nRecords done: %zu, Total: %g seconds, Avg: %g seconds\n", done + b0 + nb, t, t / (b0 + nb));
        fflush(stdout);
    }
    fclose(op);
    return 0;
}

int main(int argc, char** argv)
{
    std::vector<const char*> pos;
    bool divide = false, tt = false, records = false;
    const char* tt_load = nullptr;
    const char* tt_save = nullptr;
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "-divide")) divide = true;
        else if (!strcmp(argv[i], "-tt")) tt = true;
        else if (!strcmp(argv[i], "-records")) records = true;
        else if (!strcmp(argv[i], "-ttload") && i + 1 < argc) tt_load = argv[++i], tt = true;
        else if (!strcmp(argv[i], "-ttsave") && i + 1 < argc) tt_save = argv[++i], tt = true;
        else if (!strcmp(argv[i], "-ttmib") && i + 1 < argc) g_tt_bytes = (uint64_t)atoll(argv[++i]) << 20;
        else pos.push_back(argv[i]);
    }
    if (pg_init(nullptr) != PG_OK) return fail("pg_init");
    if (tt_load && pg_tt_load(tt_load) != PG_OK) return fail("pg_tt_load");
    auto finish = [&](int rc) {
        if (rc == 0 && tt_save && pg_tt_save(tt_save) != PG_OK) rc = fail("pg_tt_save");
        pg_shutdown();
        return rc;
    };
    if (records) {
        if (pos.empty()) {
            printf("usage: perft_gpu -records <inFile> [depth] [-tt]\n");
            return 1;
        }
        const int depth = pos.size() > 1 ? atoi(pos[1]) : 7;
        return finish(records_mode(pos[0], depth, tt));
    }
    const char* start = "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1";
    const char* fen = (!pos.empty() && strlen(pos[0]) > 5) ? pos[0] : start;
    int maxDepth = pos.size() > 1 ? atoi(pos[1]) : 3;
    if (pos.size() < 2) printf("\nUsage perft_gpu <fen> <depth> [<numGPUs>] [<launchdepth>]\n");
    if (pos.size() > 2 && atoi(pos[2]) != 1) printf("\n%s GPUs requested; this engine drives one GPU per process\n", pos[2]);
    pg_board b;
    if (pg_board_from_fen(fen, &b) != PG_OK) return fail("FEN");
    pg_opts o{};
    o.use_tt = tt ? 1 : 0;
    o.tt_bytes = g_tt_bytes;
    const int minDepth = maxDepth < 3 ? maxDepth : 3;
    for (int depth = minDepth; depth <= maxDepth; depth++) {
        const double t0 = now_s();
        if (depth >= 9 || (divide && depth == maxDepth)) {
            pg_move mv[256];
            uint64_t cnt[256];
            uint32_t n = 0;
            const int split = depth >= 9 ? 3 : 1;
            if (pg_perft_split(&b, depth, split, mv, cnt, &n, &o) != PG_OK) return fail("pg_perft_split");
            uint64_t total = 0;
            printf("\n");
            for (uint32_t i = 0; i < n; i++) {
                printf("..%s   %20llu\n", move_string(mv[i]).c_str(), (unsigned long long)cnt[i]);
                total += cnt[i];
            }
            printf("Perft(%02d):%20llu, time: %8g s\n", depth, (unsigned long long)total, now_s() - t0);
        } else {
            uint64_t res = 0;
            if (pg_perft(&b, depth, &res, &o) != PG_OK) return fail("pg_perft");
            const double t = now_s() - t0;
            printf("\nGPU Perft %d: %llu,   Time taken: %g seconds, nps: %llu\n", depth, (unsigned long long)res, t,
                   (unsigned long long)(t > 0 ? res / t : 0));
        }
        fflush(stdout);
    }
    return finish(0);
}
