/*
 * perft_gb300.h -- C ABI of the GB300 (sm_103a) perft engine.
 *
 * Drop-in surface for the perft path of sarona-RD/perft_gpu.  Types are
 * byte-identical to the reference's: pg_board is HexaBitBoardPosition
 * (chess.h:207-230, 48 bytes) and pg_move is CMove (chess.h:234-268, 16 bits:
 * from 0-5, to 6-11, flags 12-15).  Every entry point returns a pg_status
 * (0 = PG_OK) instead of printing and exiting; pg_last_error() gives the
 * message of the last failure on the calling thread.  Host arrays are owned
 * by the caller; device memory is owned by the engine.  There is no CPU
 * fallback: every count below is computed by CUDA kernels on the GPU, and
 * the calls fail with PG_ERR_CUDA when no usable GPU is present.
 *
 * Thread safety: the engine serialises calls internally; one engine per
 * process (the reference's MoveGeneratorBitboard::init is also per process,
 * MoveGeneratorBitboard.h:982).
 */
#ifndef PERFT_GB300_H
#define PERFT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* HexaBitBoardPosition (chess.h:207-230): six bitboards; the game state is
 * packed into the pawns word: bits 0-1 white castling (1 = king side,
 * 2 = queen side), bits 2-3 black castling, bits 4-7 en-passant file + 1,
 * bits 56-62 half-move counter, bit 63 side to move (0 white, 1 black). */
typedef struct pg_board {
    uint64_t white;
    uint64_t pawns;
    uint64_t knights;
    uint64_t bishop_queens;
    uint64_t rook_queens;
    uint64_t kings;
} pg_board;

/* CMove (chess.h:234-268). */
typedef uint16_t pg_move;

typedef enum pg_status {
    PG_OK = 0,
    PG_ERR_NOT_INITIALIZED = 1,
    PG_ERR_INVALID_ARGUMENT = 2,
    PG_ERR_INVALID_POSITION = 3, /* not exactly one king per side, overlapping bitboards */
    PG_ERR_CUDA = 4,
    PG_ERR_OUT_OF_MEMORY = 5,    /* HBM budget too small for the request */
    PG_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up */
    PG_ERR_BUSY = 7,
    PG_ERR_CAPACITY = 8          /* fixed-size buffer of a call exceeded */
} pg_status;

typedef enum pg_slider {
    PG_SLIDER_AUTO = 0,      /* autotuner's choice */
    PG_SLIDER_KOGGE_STONE = 1,
    PG_SLIDER_FANCY = 2,     /* fancy magics, attack table in global memory (L2) */
    PG_SLIDER_BYTE_SMEM = 3, /* byte-lookup fancy magics staged in shared memory */
    PG_SLIDER_HYBRID = 4     /* Kogge-Stone enemy fills, magic lookups for the king and own sliders */
} pg_slider;

/* pg_opts.use_tt.  PG_TT_ON: the per-depth HBM tables plus the in-level
 * duplicate pass (the reference's perft_bb_gpu_simple_hash,
 * perft_bb.h:1242-1589).  PG_TT_DEDUP_ONLY: the same driver with only the
 * duplicate pass inside each level (no HBM tables: none allocated, probed or
 * stored).  Counts are identical in every mode. */
typedef enum pg_tt_mode {
    PG_TT_OFF = 0,
    PG_TT_ON = 1,
    PG_TT_DEDUP_ONLY = 2
} pg_tt_mode;

typedef struct pg_config {
    int device;                  /* CUDA device ordinal (default 0) */
    uint64_t hbm_budget_bytes;   /* level buffers + TT; 0 = 60% of free HBM */
    int slider;                  /* default slider policy (pg_slider) */
    int verbose;
} pg_config;

typedef struct pg_stats {
    double device_ms;            /* CUDA-event time of the engine's launches */
    uint64_t leaves;             /* sum of the results */
    uint64_t launches;           /* kernels launched by the call */
    uint64_t peak_level_bytes;   /* largest frontier level held */
    uint64_t tt_probes, tt_hits, tt_stores;
    uint64_t leaf_kernel_launches;
    double leaf_kernel_ms;       /* CUDA-event time of the leaf (2-ply) kernel launches */
    uint64_t leaf_parent_nodes;  /* nodes handed to the leaf kernel (each 2 plies above a leaf) */
    uint64_t graph_captures;     /* 1 when this call captured its launch sequence into a graph */
    uint64_t graph_replays;      /* 1 when this call replayed a captured graph */
} pg_stats;

typedef struct pg_opts {
    int slider;                  /* pg_slider; PG_SLIDER_AUTO = tuned per call */
    int block_size;              /* leaf/expand CTA size: 0 = tuned, else 128/256/512 */
    int leaf_plies;              /* plies handled inside one CTA at the leaf: 0 = tuned, 1 or 2 */
    int use_tt;                  /* pg_tt_mode: PG_TT_OFF, PG_TT_ON, PG_TT_DEDUP_ONLY */
    uint64_t tt_bytes;           /* total TT bytes across depths; 0 = from budget */
    int graph;                   /* replay the call's launch sequence from a captured CUDA graph */
    pg_stats *stats;             /* optional out */
    int persistent;              /* the whole batch as one persistent cooperative launch that walks
                                    the levels and chunks on the device (Kogge-Stone sliders, 128-thread
                                    CTAs, two-ply leaf; no TT): the reference's device-side driver,
                                    perft_bb.h:1143-1220, without dynamic parallelism */
} pg_opts;

/* ---- engine ---- */
/* MoveGeneratorBitboard::init (MoveGeneratorBitboard.h:982-1203) plus the
 * allocation of initGPU (launcher.h:1506-1533). cfg may be NULL. */
int pg_init(const pg_config *cfg);
int pg_shutdown(void);
const char *pg_last_error(void);
/* Utils::readFENString + board088ToHexBB (util.cpp:189-280, util.cpp:92-140). */
int pg_board_from_fen(const char *fen, pg_board *out);
/* The CUDA stream (cudaStream_t) every engine launch is issued on, so a
 * caller can order its own work or record CUDA events around engine calls.
 * No counterpart in the reference, which launches on the default stream. */
int pg_get_stream(void **stream);

/* ---- operator surface (GPU kernels, one position per call or a batch) ---- */
/* countMoves<c> (MoveGeneratorBitboard.h:3008-3295). */
int pg_count_moves(const pg_board *pos, uint32_t *out);
int pg_count_moves_batch(const pg_board *pos, uint32_t n, uint32_t *out);
/* generateMoves<c> (MoveGeneratorBitboard.h:2469-2823), host flavour:
 * same order and flags as the reference's host build; moves holds 256. */
int pg_generate_moves(const pg_board *pos, pg_move *moves, uint32_t *n);
/* generateBoards<c> (MoveGeneratorBitboard.h:1940-2261); out holds 256. */
int pg_generate_boards(const pg_board *pos, pg_board *out, uint32_t *n);
/* makeMove<c,false> (MoveGeneratorBitboard.h:3310-3570), in place. */
int pg_make_move(pg_board *pos, pg_move move);

/* ---- perft ---- */
/* perft_bb (perft_bb.h:79-101) / perftLauncher (launcher.h:1455-1504),
 * which prints instead of returning; depth 0..15. */
int pg_perft(const pg_board *pos, int depth, uint64_t *out, const pg_opts *opts);
/* divided perft: counts[i] = perft(child after moves[i], depth-1) for every
 * legal root move in generateMoves order (perft_bb_cpu_launcher's per-move
 * lines, launcher.h:1344-1351); moves/counts hold 256. */
int pg_perft_divide(const pg_board *pos, int depth, pg_move *moves, uint64_t *counts,
                    uint32_t *n, const pg_opts *opts);
/* n positions, each with its own depth, in one load-balanced engine run.
 * Host arrays. */
int pg_perft_batch(const pg_board *pos, const uint8_t *depths, uint32_t n, uint64_t *out,
                   const pg_opts *opts);
/* The same with device pointers (inputs already resident in HBM). */
int pg_perft_batch_device(const pg_board *d_pos, const uint8_t *d_depths, uint32_t n,
                          uint64_t *d_out, const pg_opts *opts);

/* Batched perft for callers that cannot allocate device memory: a process
 * whose memory pool already owns the whole GPU, a framework allocator that
 * forbids side allocations, or code running where allocation is not
 * allowed.  No counterpart in the reference.  d_pos / d_depths / d_out are
 * device pointers owned by the caller; all working memory is one file-scope
 * device array of 60 MiB that every GPU loading this library keeps until
 * the process exits, so the call makes no cudaMalloc, cudaFree or other
 * allocating call.  Limits: n <= 65536 positions, depths 0..3, and at most
 * 1,048,576 children of the depth-3 positions per call (both sides to move
 * together).  Larger requests return PG_ERR_CAPACITY; every size check is
 * made before the counting kernels, so d_out then holds zeros.  The first
 * call on a device uploads the move tables (about 0.9 MB, into file-scope
 * device arrays of this library); make that first call before any stream
 * capture.  Every call looks up the array's device address again (no
 * allocation), and a call that finds the tables gone after a device reset
 * uploads them again.  stream may be NULL (the default stream); the call
 * synchronises it and returns when d_out is written.  Every call reuses the
 * same array, so calls that overlap on the GPU (other threads, other
 * streams) race.  Does not need pg_init. */
int pg_perft_batch_noalloc(const pg_board *d_pos, const uint8_t *d_depths, uint32_t n,
                           uint64_t *d_out, void *stream);

/* The autotuner's choices (it runs once, on the first call that leaves slider,
 * block size and switch depth at 0, or here).  Per root depth d: the slider
 * policy and CTA size of the leaf kernel and the calibration rate in leaf
 * nodes/s (depths 3..6 measured; shallower/deeper copy the ends).
 * leaf_plies is the switch depth: plies finished inside one CTA.  No
 * counterpart in the reference (its switches are compile-time, switches.h). */
typedef struct pg_tuning {
    int leaf_plies;
    int slider[16];
    int block_size[16];
    double leaves_per_s[16];
    double seconds;
} pg_tuning;
int pg_autotune(pg_tuning *out);

/* Empty the transposition tables (they persist across calls otherwise; an
 * entry stays valid for its position and remaining depth, so results never
 * depend on what earlier calls stored).  No counterpart in the reference. */
int pg_tt_clear(void);

/* The 128-bit Zobrist key the device tables use for a position
 * (computeZobristKey128b, MoveGeneratorBitboard.h:3914-3980, and
 * HashKey128b, chess.h:410-452, with this engine's seeded key set): key[0]
 * is the low word (its low bits pick the table slot), key[1] the high word.
 * The half-move clock is not part of the key.  Host code: needs no GPU and
 * no pg_init. */
int pg_zobrist_key(const pg_board *pos, uint64_t key[2]);
/* The key of pos from the key of another board `from`: from_key XOR the
 * features in which the two boards differ (for a parent and its child, the
 * squares the move changed, the castling rights and en-passant files, the
 * side to move) -- the incremental update of the reference's
 * makeMove<c, true> (MoveGeneratorBitboard.h:3575-3836), the code the probe
 * kernel runs below the root level.  Equals pg_zobrist_key(pos) whenever
 * from_key == pg_zobrist_key(from).  Host code: needs no GPU and no pg_init. */
int pg_zobrist_key_from(const pg_board *from, const uint64_t from_key[2], const pg_board *pos, uint64_t key[2]);
/* The 32-byte table entry of a key and its count, and the check a probe
 * makes (the reference's XOR-verified entries, chess.h:454-482 and the probe
 * of perft_bb.h:690-693, widened to verify all 128 key bits):
 * entry = {k0 ^ v, k1 ^ v, v, mix(k0, k1) ^ v}; pg_tt_entry_match sets
 * *accepted to 1 and *count to v only when all three checks hold for key.
 * Host code: needs no GPU and no pg_init. */
int pg_tt_entry_pack(const uint64_t key[2], uint64_t count, uint64_t entry[4]);
int pg_tt_entry_match(const uint64_t entry[4], const uint64_t key[2], int *accepted, uint64_t *count);

/* Snapshot of the transposition tables on disk, so a later process starts
 * with the subtrees an earlier one counted (the reference's disk hash,
 * launcher.h:699-790, keeps a chained table in a file instead; off there by
 * default).  pg_tt_save writes the tables as they are (a header, then the
 * tables: about the TT size in bytes); pg_tt_load reads a snapshot back,
 * making tables of the snapshot's size, and rejects files that are not
 * snapshots of this engine (format, Zobrist keys, depth range). */
int pg_tt_save(const char *path);
int pg_tt_load(const char *path);

/* Divided perft at deep roots: perft_bb_cpu_launcher (launcher.h:1181-1389)
 * with its complete transposition table (launcher.h:598-680).  The positions
 * split_plies below each root move are made on the GPU and merged across all
 * root moves in a host table keyed by the full board, so each distinct one is
 * counted once; moves/counts as pg_perft_divide (generateMoves order).
 * stats->tt_probes / tt_hits count the host table's lookups / repeats. */
int pg_perft_split(const pg_board *pos, int depth, int split_plies, pg_move *moves, uint64_t *counts,
                   uint32_t *n, const pg_opts *opts);

/* Failure-detection self tests; neither faults nor hangs the GPU.
 * PG_SELFTEST_BOUNDED_WAIT launches a scan tile whose predecessor never
 * publishes: its poll gives up after the limit and the call returns
 * PG_ERR_DEVICE_TIMEOUT, with the context still usable.
 * PG_SELFTEST_FAIL_NEXT_ALLOC makes the next level allocation fail on the
 * host, so the following call returns PG_ERR_OUT_OF_MEMORY and the one after
 * it works.  No counterpart in the reference. */
enum { PG_SELFTEST_BOUNDED_WAIT = 1, PG_SELFTEST_FAIL_NEXT_ALLOC = 2 };
int pg_selftest(int which);

/* ---- inputs ---- */
/* Seeded random legal playouts from the initial position, generated on the
 * GPU.  Position i is the first accepted attempt a = 0, 1, ... of:
 * s = seed ^ (i << 32) ^ (a * 0xA24BAED4963EE407); plies = min_plies +
 * next(s) % (max_plies - min_plies + 1); per ply pick
 * generateMoves[next(s) % count] and makeMove; accepted when every ply had a
 * move and the final position has at least min_moves legal moves.  next() is
 * splitmix64.  depths (may be NULL): depth_lo + next(s') % (depth_hi -
 * depth_lo + 1) with s' = seed ^ (i << 32) ^ 0x5851F42D4C957F2D. */
int pg_random_playouts(uint64_t seed, uint32_t n, int min_plies, int max_plies, int min_moves,
                       int depth_lo, int depth_hi, pg_board *out, uint8_t *depths);

/* ---- serving: continuous batching of perft requests ---- */
typedef struct pg_server_config {
    uint64_t hbm_budget_bytes;   /* admission budget for in-flight frontiers; 0 = 2 GiB */
    uint32_t max_inflight;       /* request slots; 0 = 4096 */
    int slider;
    uint32_t max_wave_nodes;     /* fixed wave size in frontier nodes (positions 5 plies above the
                                    leaves); 0 = waves sized in time, about 4 ms of device work
                                    each from the measured rate and leaves per task */
    int use_tt;                  /* pg_tt_mode of the waves; with PG_TT_ON the tables persist
                                    across requests (launcher.h:699-790 keeps its table across runs) */
    uint64_t tt_bytes;           /* TT size when use_tt; 0 = from the engine budget (as pg_opts) */
    int persistent;              /* run each wave (without TT) as one persistent launch (pg_opts.persistent) */
} pg_server_config;

int pg_server_start(const pg_server_config *cfg);
/* Returns at once with a request id; the request joins the running waves. */
int pg_server_submit(const pg_board *pos, int depth, uint64_t *request_id);
/* done = 1 once the count is final; latency_ms from submit to completion. */
int pg_server_poll(uint64_t request_id, uint64_t *result, int *done, double *latency_ms);
int pg_server_stop(void);
/* Counters of the running server.  admissions_deferred counts the times the
 * first waiting request did not fit the free frontier pool while others ran
 * (it is then admitted first once a free block holds what it needs);
 * pool_capacity / pool_peak are in positions (48 bytes each). */
typedef struct pg_server_stats {
    uint64_t submitted, completed, waves;
    uint64_t admissions_deferred;
    uint32_t max_active;         /* most requests in flight at once */
    uint64_t pool_capacity, pool_peak;
} pg_server_stats;
int pg_server_get_stats(pg_server_stats *out);

#ifdef __cplusplus
}
#endif
#endif
