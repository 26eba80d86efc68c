/*
 * gal_oracle.h — CPU restatement of the reference allocator's single-thread
 * semantics (chillenzer/gallatin, include/gallatin/allocators/ headers).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load this; the product never does.
 *
 * Parity: pinned against the reference's own CUDA build (compiled from its
 * sources into oracle/_ref/ and run on a GB300; fixtures in tests/golden/).
 */
#ifndef GAL_ORACLE_H
#define GAL_ORACLE_H

#include <stdint.h>
#include "../include/gallatin_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_FAIL (~0ULL)

/* Behaviour switches.  0 = exactly the reference.  The product fixes the
 * listed reference defects; the oracle models either side. */
#define ORC_FIX_GATHER_EXIT_ROLLBACK 0x1u /* veb.cuh:447 spurious rollback   */
/* block.cuh:267-281 adds a malloc's leftover slices to the free counter with
 * no completion check; when those slices are the last ones the block was
 * owed, the block is never returned (leaked).  With the fix the leftover
 * credit completes the block like any other free. */
#define ORC_FIX_LEFTOVER_COMPLETES 0x2u
/* veb.cuh:382-410: a run that still needs more than the words below it
 * steps to word -1.  With the fix the request fails and the words it took
 * (word 0 up to its first word) are given back. */
#define ORC_FIX_RUN_BELOW_ARENA 0x4u
/* veb.cuh:1128-1154: returning a run lists a bottom word in the summary only
 * when the word is then full.  A run whose claim emptied its first or last
 * word gives that word back partly filled and unlisted, so the single-item
 * searches never reach its segments again (nor does a later insert into the
 * word, which climbs only from an empty word).  With the fix every word the
 * run leaves non-empty is listed. */
#define ORC_FIX_RUN_RETURN_SUMMARY 0x8u

typedef struct orc_alloc orc_alloc;

orc_alloc *orc_create(uint64_t num_bytes, uint64_t seed, uint64_t bytes_per_segment,
                      uint64_t min_size, uint64_t max_size, uint32_t pinned_first,
                      uint32_t pinned_min, uint32_t fix_flags, uint32_t policy);
void orc_destroy(orc_alloc *a);

/* model the product's spare blocks (gal_config.spare_blocks = 1) */
void orc_set_spares(orc_alloc *a, int on);

/* boot_shared_block_container_one_thread (gallatin.cuh:196-221), thread id 0 */
int orc_boot_one_thread(orc_alloc *a);

/* retire every pinned block, then boot the slots again (gal_trim) */
int orc_trim(orc_alloc *a);

/* device malloc/free of one thread; offsets are byte offsets from the arena
 * base, ORC_FAIL for nullptr. */
uint64_t orc_malloc(orc_alloc *a, uint64_t size, uint32_t smid, uint64_t tid);
void orc_free(orc_alloc *a, uint64_t byte_offset);

/* replay a trace (encoding as gal_replay_trace); returns 0 */
int orc_replay(orc_alloc *a, const uint64_t *ops, uint64_t nops, uint32_t smid,
               uint64_t tid, uint64_t *out_offsets);

/* replay a trace of warp-wide calls by one warp (encoding as
 * gal_replay_warp_trace); returns 0, -1 for a malformed step */
int orc_replay_warp(orc_alloc *a, const uint64_t *steps, uint64_t nsteps, uint32_t smid,
                    uint64_t tid0, uint64_t *out);

int orc_dims(orc_alloc *a, gal_state_dims *out);
int orc_export(orc_alloc *a, const gal_state_view *v);
int orc_import(orc_alloc *a, const gal_state_view *v);

/* serial trace generator (splitmix64), see oracle/gal_oracle.c */
int orc_gen_serial_trace(uint64_t seed, uint64_t nops, uint32_t malloc_pct,
                         uint64_t size_quantum, uint64_t size_steps, uint64_t *ops);

int orc_gen_trace_log(uint64_t seed, uint64_t nops, uint32_t malloc_pct, uint32_t lo_bits,
                      uint32_t hi_bits, uint64_t *ops);

uint64_t orc_murmur64a_u64(uint64_t key, uint64_t seed);
uint64_t orc_arena_bytes(orc_alloc *a);

#ifdef __cplusplus
}
#endif
#endif
