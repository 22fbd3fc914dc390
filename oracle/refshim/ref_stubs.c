/*
 * Link stubs for compiling the reference hot-path sources as the oracle
 * (TEST INFRASTRUCTURE ONLY). They replace the engine services those files
 * call: the clock (src/ctx.c:114-116), logging and panic (src/event.c), and
 * the labelled heap (src/mem.c). Allocations are over-sized (4x + 64 bytes)
 * because rle_compress sizes its word buffer in bytes but writes u32 words
 * (src/chunkset/rle.c:49).
 */
#include <stdlib.h>
#include <stddef.h>

double ctx_time(void) { return 0.0; }
void _log_info(char *s) { (void)s; }
void _log_warn(char *s) { (void)s; }
void _log_error(char *s) { (void)s; }
void panic(void) { abort(); }
void event_fire(int e, void *a) { (void)e; (void)a; }
void *_mem_alloc(size_t s, char *label) { (void)label; return calloc(4 * s + 64, 1); }
void *_mem_calloc(size_t s, char *label) { (void)label; return calloc(4 * s + 64, 1); }
void *_mem_free(void *p, char *label) { (void)label; free(p); return NULL; }
size_t mem_dynamic_allocation(void) { return 0; }
