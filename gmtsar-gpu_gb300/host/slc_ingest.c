/* Pipelined SLC ingest for the xcorr program.
 *
 * The reference re-reads npy whole lines of both SLCs for every strip of
 * locations (read_xcorr_data.c:52-85, called per strip at xcorr.cu:326-328),
 * converts them to float on the host and copies one patch at a time
 * (xcorr.cu:336-337).  Here each needed line is read once: a reader thread
 * streams bands of lines of both images into pinned buffers, the main thread
 * copies each band into the device images as raw 32-bit samples (converted on
 * the GPU inside the row kernel) and launches the correlation of every strip
 * whose lines have all arrived, so reading, copying and correlating overlap.
 * Results are identical to one call over all locations: strips are never
 * split between calls. */
#define _GNU_SOURCE
#include <cuda_runtime.h>
#include <fcntl.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "xcorr_cli.h"

#define NSLOT 3

typedef struct {
    int fd[2];
    int nx[2], ny[2];
    int row0[2];               /* first line read of each image */
    int band;                  /* lines per band */
    int nbands;
    unsigned char *buf[NSLOT][2];
    int ready[NSLOT];          /* band index held by the slot, -1: empty */
    int stop;
    pthread_mutex_t mu;
    pthread_cond_t cv;
} ingest;

static void read_lines(int fd, unsigned char *dst, int nx, int ny, int y0, int n)
{
    const size_t line = (size_t)nx * 4;
    size_t want = (size_t)n * line, got = 0;
    if (y0 < ny) {
        off_t pos = (off_t)y0 * (off_t)line;
        size_t avail = (size_t)(ny - y0) * line;
        size_t todo = want < avail ? want : avail;
        while (got < todo) {
            ssize_t r = pread(fd, dst + got, todo - got, pos + (off_t)got);
            if (r <= 0) break;       /* short file: the rest stays zero */
            got += (size_t)r;
        }
    }
    if (got < want) memset(dst + got, 0, want - got);
}

static void *reader(void *arg)
{
    ingest *g = (ingest *)arg;
    for (int b = 0; b < g->nbands; b++) {
        const int slot = b % NSLOT;
        pthread_mutex_lock(&g->mu);
        while (g->ready[slot] != -1 && !g->stop) pthread_cond_wait(&g->cv, &g->mu);
        const int stop = g->stop;
        pthread_mutex_unlock(&g->mu);
        if (stop) break;
        for (int k = 0; k < 2; k++) {
            int y0 = g->row0[k] + b * g->band;
            int n = g->band;
            if (y0 + n > g->ny[k]) n = g->ny[k] - y0;
            if (n > 0) read_lines(g->fd[k], g->buf[slot][k], g->nx[k], g->ny[k], y0, n);
        }
        pthread_mutex_lock(&g->mu);
        g->ready[slot] = b;
        pthread_cond_broadcast(&g->cv);
        pthread_mutex_unlock(&g->mu);
    }
    return NULL;
}

/* on a CUDA error: report it, and leave through the cleanup below */
#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            fprintf(stderr, "xcorr: %s: %s\n", #call, cudaGetErrorString(e_));    \
            failed = 1;                                                           \
            goto cleanup;                                                         \
        }                                                                         \
    } while (0)

int xcli_correlate_streamed(const xcli *xc, xcg_ctx *ctx, xcg_result *host_results)
{
    const int ns = xc->nyl, nxl = xc->nxl, npy = xc->npy;
    if (xc->nlocs == 0) return 0;
    int failed = 0, started = 0;
    ingest g;
    memset(&g, 0, sizeof g);
    g.fd[0] = g.fd[1] = -1;
    void *d_img[2] = {NULL, NULL};
    xcg_loc *d_locs = NULL;
    xcg_result *d_res = NULL;
    cudaStream_t st = NULL;
    cudaEvent_t ev = NULL;
    pthread_t th;
    /* lines each strip needs (exclusive end) and the first line anyone needs */
    int *need[2];
    need[0] = (int *)malloc(sizeof(int) * (size_t)ns);
    need[1] = (int *)malloc(sizeof(int) * (size_t)ns);
    int first[2] = {1 << 30, 1 << 30};
    for (int s = 0; s < ns; s++) {
        need[0][s] = need[1][s] = 0;
        for (int i = s * nxl; i < (s + 1) * nxl && i < xc->nlocs; i++) {
            const int y = xc->loc[i].y;
            const int ishft = (int)(y * xc->astretcha);
            const int ym = y - npy / 2, ys = y + xc->y_offset + ishft - npy / 2;
            if (ym + npy > need[0][s]) need[0][s] = ym + npy;
            if (ys + npy > need[1][s]) need[1][s] = ys + npy;
            if (ym < first[0]) first[0] = ym;
            if (ys < first[1]) first[1] = ys;
        }
    }
    const char *names[2] = {xc->data1_name, xc->data2_name};
    g.nx[0] = xc->m_nx; g.ny[0] = xc->m_ny;
    g.nx[1] = xc->s_nx; g.ny[1] = xc->s_ny;
    g.band = 256;
    int total = 0;
    for (int k = 0; k < 2; k++) {
        g.fd[k] = open(names[k], O_RDONLY);
        if (g.fd[k] < 0) xcli_die("Cannot open SLC_file", names[k]);
        g.row0[k] = first[k] < 0 ? 0 : (first[k] > g.ny[k] ? g.ny[k] : first[k]);
        const int rows = g.ny[k] - g.row0[k];
        const int nb = (rows + g.band - 1) / g.band;
        if (nb > total) total = nb;
    }
    g.nbands = total;
    pthread_mutex_init(&g.mu, NULL);
    pthread_cond_init(&g.cv, NULL);
    for (int s = 0; s < NSLOT; s++) {
        g.ready[s] = -1;
        for (int k = 0; k < 2; k++) CK(cudaMallocHost((void **)&g.buf[s][k], (size_t)g.band * g.nx[k] * 4));
    }
    CK(cudaMalloc(&d_img[0], (size_t)g.nx[0] * g.ny[0] * 4));
    CK(cudaMalloc(&d_img[1], (size_t)g.nx[1] * g.ny[1] * 4));
    CK(cudaMalloc((void **)&d_locs, sizeof(xcg_loc) * (size_t)xc->nlocs));
    CK(cudaMalloc((void **)&d_res, sizeof(xcg_result) * (size_t)xc->nlocs));
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaMemcpyAsync(d_locs, xc->loc, sizeof(xcg_loc) * (size_t)xc->nlocs, cudaMemcpyHostToDevice, st));

    pthread_create(&th, NULL, reader, &g);
    started = 1;
    int next = 0;
    for (int b = 0; b <= g.nbands && !failed; b++) {
        int avail[2];
        if (b < g.nbands) {
            const int slot = b % NSLOT;
            pthread_mutex_lock(&g.mu);
            while (g.ready[slot] != b) pthread_cond_wait(&g.cv, &g.mu);
            pthread_mutex_unlock(&g.mu);
            for (int k = 0; k < 2; k++) {
                const int y0 = g.row0[k] + b * g.band;
                int n = g.band;
                if (y0 + n > g.ny[k]) n = g.ny[k] - y0;
                if (n > 0)
                    CK(cudaMemcpyAsync((unsigned char *)d_img[k] + (size_t)y0 * g.nx[k] * 4, g.buf[slot][k],
                                       (size_t)n * g.nx[k] * 4, cudaMemcpyHostToDevice, st));
                avail[k] = y0 + (n > 0 ? n : 0);
            }
            CK(cudaEventRecord(ev, st));
            CK(cudaEventSynchronize(ev));            /* the slot may be refilled; kernels keep running */
            pthread_mutex_lock(&g.mu);
            g.ready[slot] = -1;
            pthread_cond_broadcast(&g.cv);
            pthread_mutex_unlock(&g.mu);
        } else {
            avail[0] = 1 << 30;                      /* everything is in */
            avail[1] = 1 << 30;
        }
        /* a strip is ready once every line it reads inside its images is in;
         * lines past an image's end are zero-filled by the row kernel */
        int last = next;
        while (last < ns && (need[0][last] < g.ny[0] ? need[0][last] : g.ny[0]) <= avail[0] &&
               (need[1][last] < g.ny[1] ? need[1][last] : g.ny[1]) <= avail[1])
            last++;
        if (last > next) {
            const int w0 = next * nxl;
            int w1 = last * nxl;
            if (w1 > xc->nlocs) w1 = xc->nlocs;
            xcg_status s = xcg_correlate_device(ctx, d_img[0], g.nx[0], g.ny[0], d_img[1], g.nx[1], g.ny[1],
                                                xc->x_offset, xc->y_offset, xc->astretcha, d_locs + w0, w1 - w0,
                                                nxl, d_res + w0, st);
            if (s != XCG_OK) {
                fprintf(stderr, "xcorr: %s: %s\n", xcg_status_string(s), xcg_last_error());
                failed = 1;
            }
            next = last;
        }
    }
    if (!failed) {
        CK(cudaMemcpyAsync(host_results, d_res, sizeof(xcg_result) * (size_t)xc->nlocs, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
cleanup:
    if (started) {
        pthread_mutex_lock(&g.mu);
        g.stop = 1;
        pthread_cond_broadcast(&g.cv);
        pthread_mutex_unlock(&g.mu);
        pthread_join(th, NULL);
    }
    if (st) cudaStreamSynchronize(st);
    for (int s = 0; s < NSLOT; s++)
        for (int k = 0; k < 2; k++)
            if (g.buf[s][k]) cudaFreeHost(g.buf[s][k]);
    cudaFree(d_img[0]); cudaFree(d_img[1]); cudaFree(d_locs); cudaFree(d_res);
    if (ev) cudaEventDestroy(ev);
    if (st) cudaStreamDestroy(st);
    for (int k = 0; k < 2; k++)
        if (g.fd[k] >= 0) close(g.fd[k]);
    free(need[0]); free(need[1]);
    return failed;
}
