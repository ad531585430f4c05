/* pvvc_oracle_zstd.c -- test and benchmark infrastructure, not shipped.
 *
 * libzstd's ZSTD_decompress over a batch of payloads on host threads: the
 * reference's own zstd stage (ZstdDecoder::Decode, src/common/entropy_codec.cc:
 * 341-360, which io::LoadFrame runs on every zstd payload,
 * src/cuda/common/slice_io.cu:233-265).  Timed as the CPU baseline of the
 * GPU inflater.  libzstd is loaded at run time (libzstd.so.1). */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#include "pvvc_oracle.h"

typedef size_t (*zdec_fn)(void*, size_t, const void*, size_t);
typedef unsigned (*zerr_fn)(size_t);

typedef struct {
    zdec_fn dec;
    zerr_fn err;
    const uint8_t* src;
    const uint64_t* src_off;
    const uint32_t* src_len;
    uint8_t* dst;
    const uint64_t* dst_off;
    const uint32_t* dst_cap;
    int32_t* status;
    int n, nthreads, t;
} zjob;

static void* zworker(void* arg) {
    zjob* j = (zjob*)arg;
    for (int i = j->t; i < j->n; i += j->nthreads) {
        const size_t r = j->dec(j->dst + j->dst_off[i], j->dst_cap[i], j->src + j->src_off[i], j->src_len[i]);
        j->status[i] = j->err(r) ? 9 : 0;
    }
    return NULL;
}

int pvo_libzstd_inflate_batch(int n, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len, uint8_t* dst,
                              const uint64_t* dst_off, const uint32_t* dst_cap, int32_t* status, int nthreads) {
    void* h = dlopen("libzstd.so.1", RTLD_NOW);
    if (!h) return -1;
    zdec_fn dec = (zdec_fn)dlsym(h, "ZSTD_decompress");
    zerr_fn err = (zerr_fn)dlsym(h, "ZSTD_isError");
    if (!dec || !err) return -1;
    if (nthreads < 1) nthreads = 1;
    zjob* jobs = (zjob*)malloc((size_t)nthreads * sizeof(zjob));
    pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        zjob j = {dec, err, src, src_off, src_len, dst, dst_off, dst_cap, status, n, nthreads, t};
        jobs[t] = j;
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, zworker, &jobs[t]);
    zworker(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    return 0;
}
