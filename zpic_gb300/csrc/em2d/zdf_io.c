/*
 * zdf_io.c -- ZDF diagnostic files for libzpic_em2d (include/em2d/zdf.h).
 *
 * Writes the record stream of ZPIC's ZDF version 1 (reference em2d/zdf.c):
 * magic "ZDF1", then records of uint32 id/version, name string, uint64
 * payload length and payload.  Strings are a uint32 length plus the bytes,
 * zero-padded to a multiple of 4.  Numbers are written little endian
 * whatever the host's byte order, composed byte by byte.
 *
 * The report calls of libzpic_em2d hand their files to one background
 * thread (zdf_async_submit), so that the simulation goes on while a file
 * is formatted and written; zdf_flush waits for the queue to drain.
 */
#define _POSIX_C_SOURCE 200809L
#define _FILE_OFFSET_BITS 64

#include <errno.h>
#include <inttypes.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "../../../include/em2d/zdf.h"

#define EXPORT __attribute__((visibility("default")))

/* record ids (id << 16 | version) */
enum {
    REC_INT32 = 0x00010000,
    REC_DOUBLE = 0x00020000,
    REC_STRING = 0x00030000,
    REC_DATASET = 0x00100002,
    REC_CDSET_START = 0x00110000,
    REC_CDSET_CHUNK = 0x00120000,
    REC_CDSET_END = 0x00130000,
    REC_ITERATION = 0x00200001,
    REC_GRID_INFO = 0x00210001,
    REC_PART_INFO = 0x00220002,
    REC_TRACK_INFO = 0x00230001
};

static size_t pad4(size_t n) { return (n + 3) / 4 * 4; }

/* ------------------------------------------------------------------------- */
/* little-endian scalars and vectors                                         */
/* ------------------------------------------------------------------------- */
static size_t put_bytes(t_zdf_file *f, const void *p, size_t n)
{
    return (n == 0 || fwrite(p, 1, n, f->fp) == n) ? n : 0;
}

static size_t put_u32(t_zdf_file *f, uint32_t v)
{
    unsigned char b[4];
    for (int i = 0; i < 4; i++) b[i] = (unsigned char)(v >> (8 * i));
    return put_bytes(f, b, 4);
}

static size_t put_u64(t_zdf_file *f, uint64_t v)
{
    unsigned char b[8];
    for (int i = 0; i < 8; i++) b[i] = (unsigned char)(v >> (8 * i));
    return put_bytes(f, b, 8);
}

static size_t put_f64(t_zdf_file *f, double d)
{
    uint64_t v;
    memcpy(&v, &d, 8);
    return put_u64(f, v);
}

static int host_is_little(void)
{
    const uint16_t one = 1;
    unsigned char c;
    memcpy(&c, &one, 1);
    return c == 1;
}

/* n elements of `width` bytes each; 8-bit data is padded to 4 bytes */
static size_t put_vector(t_zdf_file *f, const void *data, size_t width, size_t n)
{
    if (width == 1) {
        if (!put_bytes(f, data, n)) return n ? 0 : 0;
        const unsigned char zero[4] = {0, 0, 0, 0};
        const size_t np = pad4(n) - n;
        if (np && !put_bytes(f, zero, np)) return 0;
        return pad4(n);
    }
    if (host_is_little()) return put_bytes(f, data, width * n) == width * n ? width * n : 0;
    unsigned char buf[4096];
    const unsigned char *src = (const unsigned char *)data;
    const size_t per = sizeof(buf) / width;
    for (size_t i0 = 0; i0 < n; i0 += per) {
        const size_t m = (n - i0 < per) ? n - i0 : per;
        for (size_t i = 0; i < m; i++)
            for (size_t b = 0; b < width; b++) buf[i * width + b] = src[(i0 + i) * width + (width - 1 - b)];
        if (!put_bytes(f, buf, m * width)) return 0;
    }
    return width * n;
}

static size_t string_size(const char *s)
{
    const size_t n = s ? strlen(s) : 0;
    return 4 + (n ? pad4(n) : 0);
}

static size_t put_string(t_zdf_file *f, const char *s)
{
    const size_t n = s ? strlen(s) : 0;
    if (!put_u32(f, (uint32_t)n)) return 0;
    if (n && !put_vector(f, s, 1, n)) return 0;
    return string_size(s);
}

static size_t put_record(t_zdf_file *f, uint32_t id, const char *name, uint64_t length)
{
    if (!put_u32(f, id)) return 0;
    const size_t ns = put_string(f, name);
    if (!ns) return 0;
    if (!put_u64(f, length)) return 0;
    return 4 + ns + 8;
}

/* ------------------------------------------------------------------------- */
/* files                                                                     */
/* ------------------------------------------------------------------------- */
EXPORT size_t zdf_sizeof(enum zdf_data_type t)
{
    switch (t) {
    case zdf_int8:
    case zdf_uint8:
        return 1;
    case zdf_int16:
    case zdf_uint16:
        return 2;
    case zdf_int32:
    case zdf_uint32:
    case zdf_float32:
        return 4;
    case zdf_int64:
    case zdf_uint64:
    case zdf_float64:
        return 8;
    default:
        return 0;
    }
}

EXPORT int zdf_open_file(t_zdf_file *zdf, const char *filename, enum zdf_file_access_mode mode)
{
    static const char magic[ZDF_MAGIC_LENGTH] = {'Z', 'D', 'F', '1'};
    zdf->mode = mode;
    zdf->ndatasets = 0;
    if (mode != ZDF_CREATE) {
        /* this library writes diagnostics; reading is left to the analysis tools */
        fprintf(stderr, "(*error*) zdf_open_file: only ZDF_CREATE is supported.\n");
        return 0;
    }
    zdf->fp = fopen(filename, "w+b");
    if (!zdf->fp) {
        perror("(*error*) Unable to open ZDF file for writing");
        return 0;
    }
    if (!put_bytes(zdf, magic, ZDF_MAGIC_LENGTH)) {
        fprintf(stderr, "(*error*) Unable to write magic number to ZDF file.\n");
        zdf_close_file(zdf);
        return 0;
    }
    return 1;
}

EXPORT int zdf_close_file(t_zdf_file *zdf)
{
    if (!zdf->fp) return 0;
    const int bad = fclose(zdf->fp);
    zdf->fp = NULL;
    if (bad) {
        perror("(*error*) Unable to close ZDF file");
        return 0;
    }
    return 1;
}

EXPORT size_t zdf_vector_write(t_zdf_file *zdf, const void *data, enum zdf_data_type t, size_t len)
{
    const size_t w = zdf_sizeof(t);
    if (!w) {
        fprintf(stderr, "(*error*) zdf_vector_write: Unsupported datatype.\n");
        return 0;
    }
    return put_vector(zdf, data, w, len);
}

/* ------------------------------------------------------------------------- */
/* records                                                                   */
/* ------------------------------------------------------------------------- */
EXPORT size_t zdf_add_string(t_zdf_file *zdf, const char *name, const char *str)
{
    const size_t h = put_record(zdf, REC_STRING, name, string_size(str));
    if (!h || !put_string(zdf, str)) return 0;
    return h + string_size(str);
}

EXPORT size_t zdf_add_int32(t_zdf_file *zdf, const char *name, const int32_t value)
{
    const size_t h = put_record(zdf, REC_INT32, name, 4);
    if (!h || !put_u32(zdf, (uint32_t)value)) return 0;
    return h + 4;
}

EXPORT size_t zdf_add_double(t_zdf_file *zdf, const char *name, const double value)
{
    const size_t h = put_record(zdf, REC_DOUBLE, name, 8);
    if (!h || !put_f64(zdf, value)) return 0;
    return h + 8;
}

EXPORT size_t zdf_add_iteration(t_zdf_file *zdf, const t_zdf_iteration *it)
{
    const size_t len = 4 + 8 + string_size(it->time_units);
    const size_t h = put_record(zdf, REC_ITERATION, it->name, len);
    if (!h || !put_u32(zdf, (uint32_t)it->n) || !put_f64(zdf, it->t) || !put_string(zdf, it->time_units)) return 0;
    return h + len;
}

static size_t grid_info_size(const t_zdf_grid_info *g)
{
    size_t n = 4 + (size_t)g->ndims * 8 + string_size(g->label) + string_size(g->units) + 4;
    if (g->axis)
        for (unsigned i = 0; i < g->ndims; i++)
            n += string_size(g->axis[i].name) + 4 + 16 + string_size(g->axis[i].label) +
                 string_size(g->axis[i].units);
    return n;
}

EXPORT size_t zdf_add_grid_info(t_zdf_file *zdf, const t_zdf_grid_info *g)
{
    const size_t len = grid_info_size(g);
    const size_t h = put_record(zdf, REC_GRID_INFO, g->name, len);
    if (!h || !put_u32(zdf, g->ndims)) return 0;
    for (unsigned i = 0; i < g->ndims; i++)
        if (!put_u64(zdf, g->count[i])) return 0;
    if (!put_string(zdf, g->label) || !put_string(zdf, g->units)) return 0;
    if (!put_u32(zdf, g->axis ? 1u : 0u)) return 0;
    if (g->axis) {
        for (unsigned i = 0; i < g->ndims; i++) {
            const t_zdf_grid_axis *a = &g->axis[i];
            if (!put_string(zdf, a->name) || !put_u32(zdf, (uint32_t)a->type) || !put_f64(zdf, a->min) ||
                !put_f64(zdf, a->max) || !put_string(zdf, a->label) || !put_string(zdf, a->units))
                return 0;
        }
    }
    return h + len;
}

static size_t quant_lists_size(uint32_t nq, char **q, char **l, char **u)
{
    size_t n = 0;
    for (uint32_t i = 0; i < nq; i++) n += string_size(q[i]) + string_size(l[i]) + string_size(u[i]);
    return n;
}

static int put_quant_lists(t_zdf_file *zdf, uint32_t nq, char **q, char **l, char **u)
{
    for (uint32_t i = 0; i < nq; i++)
        if (!put_string(zdf, q[i])) return 0;
    for (uint32_t i = 0; i < nq; i++)
        if (!put_string(zdf, l[i])) return 0;
    for (uint32_t i = 0; i < nq; i++)
        if (!put_string(zdf, u[i])) return 0;
    return 1;
}

EXPORT size_t zdf_add_part_info(t_zdf_file *zdf, const t_zdf_part_info *p)
{
    const size_t len = string_size(p->label) + 8 + 4 + quant_lists_size(p->nquants, p->quants, p->qlabels, p->qunits);
    const size_t h = put_record(zdf, REC_PART_INFO, p->name, len);
    if (!h || !put_string(zdf, p->label) || !put_u64(zdf, p->np) || !put_u32(zdf, p->nquants)) return 0;
    if (!put_quant_lists(zdf, p->nquants, p->quants, p->qlabels, p->qunits)) return 0;
    return h + len;
}

EXPORT size_t zdf_add_track_info(t_zdf_file *zdf, const t_zdf_track_info *t)
{
    const size_t len = string_size(t->label) + 4 * 4 + quant_lists_size(t->nquants, t->quants, t->qlabels, t->qunits);
    const size_t h = put_record(zdf, REC_TRACK_INFO, t->name, len);
    if (!h || !put_string(zdf, t->label) || !put_u32(zdf, t->ntracks) || !put_u32(zdf, t->ndump) ||
        !put_u32(zdf, t->niter) || !put_u32(zdf, t->nquants))
        return 0;
    if (!put_quant_lists(zdf, t->nquants, t->quants, t->qlabels, t->qunits)) return 0;
    return h + len;
}

/* the dataset header: uint32 id, int32 type, uint32 ndims, uint64 counts */
static size_t dataset_header_size(const t_zdf_dataset *d) { return 12 + (size_t)d->ndims * 8; }

static size_t put_dataset_header(t_zdf_file *zdf, t_zdf_dataset *d)
{
    const off_t pos = ftello(zdf->fp);
    if (pos < 0) return 0;
    d->offset = (uint64_t)pos;
    if (!put_u32(zdf, (uint32_t)d->id) || !put_u32(zdf, (uint32_t)d->data_type) || !put_u32(zdf, d->ndims)) return 0;
    for (unsigned i = 0; i < d->ndims; i++)
        if (!put_u64(zdf, d->count[i])) return 0;
    return dataset_header_size(d);
}

static uint64_t elements(const uint64_t *count, uint32_t ndims)
{
    uint64_t n = 1;
    for (uint32_t i = 0; i < ndims; i++) n *= count[i];
    return n;
}

EXPORT size_t zdf_add_dataset(t_zdf_file *zdf, t_zdf_dataset *d)
{
    const uint64_t n = elements(d->count, d->ndims);
    const size_t len = zdf_sizeof(d->data_type) * n + dataset_header_size(d);
    const size_t h = put_record(zdf, REC_DATASET, d->name, len);
    if (!h) return 0;
    d->id = ++zdf->ndatasets;
    if (!put_dataset_header(zdf, d)) return 0;
    if (n && !zdf_vector_write(zdf, d->data, d->data_type, n)) return 0;
    return h + len;
}

EXPORT size_t zdf_start_cdset(t_zdf_file *zdf, t_zdf_dataset *d)
{
    const size_t h = put_record(zdf, REC_CDSET_START, d->name, dataset_header_size(d));
    if (!h) return 0;
    d->id = ++zdf->ndatasets;
    const size_t b = put_dataset_header(zdf, d);
    return b ? h + b : 0;
}

EXPORT size_t size_zdf_chunk_header(const t_zdf_dataset *d)
{
    /* the record: id, a 16-byte name ("<id:08x>-chunk"), the length; then
     * the dataset id and count, start, stride per dimension */
    return 4 + (4 + 16) + 8 + 4 + 3 * (size_t)d->ndims * 8;
}

EXPORT size_t zdf_write_chunk_header(t_zdf_file *zdf, t_zdf_dataset *d, t_zdf_chunk *c)
{
    char name[16];
    snprintf(name, sizeof(name), "%08" PRIx64 "-chunk", d->id);
    const size_t body = 4 + 3 * (size_t)d->ndims * 8;
    const size_t len = zdf_sizeof(d->data_type) * elements(c->count, d->ndims) + body;
    const size_t h = put_record(zdf, REC_CDSET_CHUNK, name, len);
    if (!h || !put_u32(zdf, (uint32_t)d->id)) return 0;
    for (unsigned i = 0; i < d->ndims; i++)
        if (!put_u64(zdf, c->count[i])) return 0;
    for (unsigned i = 0; i < d->ndims; i++)
        if (!put_u64(zdf, c->start[i])) return 0;
    for (unsigned i = 0; i < d->ndims; i++)
        if (!put_u64(zdf, c->stride[i])) return 0;
    return h + body;
}

EXPORT size_t zdf_write_cdset(t_zdf_file *zdf, t_zdf_dataset *d, t_zdf_chunk *c)
{
    const size_t h = zdf_write_chunk_header(zdf, d, c);
    if (!h) return 0;
    const uint64_t n = elements(c->count, d->ndims);
    const size_t v = n ? zdf_vector_write(zdf, c->data, d->data_type, n) : 0;
    if (n && !v) return 0;
    return h + v;
}

EXPORT size_t zdf_end_cdset(t_zdf_file *zdf, t_zdf_dataset *d)
{
    char name[16];
    snprintf(name, sizeof(name), "%08" PRIx64 "-end", d->id);
    return put_record(zdf, REC_CDSET_END, name, 0);
}

/* ------------------------------------------------------------------------- */
/* grid and particle files                                                   */
/* ------------------------------------------------------------------------- */

/* mkdir -p (0755); an existing directory is fine */
static int make_path(const char *path)
{
    if (!path || !*path) return 0;
    if (mkdir(path, 0755) == 0 || errno == EEXIST) return 0;
    if (errno != ENOENT) return errno;
    char up[1024];
    snprintf(up, sizeof(up), "%s", path);
    char *slash = strrchr(up, '/');
    if (!slash || slash == up) return ENOENT;
    *slash = 0;
    const int e = make_path(up);
    if (e) return e;
    return (mkdir(path, 0755) == 0 || errno == EEXIST) ? 0 : errno;
}

EXPORT int zdf_open_grid_file(t_zdf_file *zdf, const t_zdf_grid_info *info, const t_zdf_iteration *it,
                              char const path[])
{
    char fn[1024];
    make_path(path);
    snprintf(fn, sizeof(fn), "%s/%s-%06u.zdf", path, info->name, (unsigned)it->n);
    if (!zdf_open_file(zdf, fn, ZDF_CREATE)) {
        fprintf(stderr, "(*error*) Unable to open ZDF file, aborting.\n");
        return 0;
    }
    if (!zdf_add_string(zdf, "TYPE", "grid") || !zdf_add_grid_info(zdf, info) || !zdf_add_iteration(zdf, it)) {
        zdf_close_file(zdf);
        return 0;
    }
    return 1;
}

EXPORT int zdf_save_grid(const void *data, enum zdf_data_type t, const t_zdf_grid_info *info,
                         const t_zdf_iteration *it, char const path[])
{
    t_zdf_file zdf;
    if (!zdf_open_grid_file(&zdf, info, it, path)) return 0;
    t_zdf_dataset d;
    memset(&d, 0, sizeof(d));
    d.name = info->name;
    d.data_type = t;
    d.ndims = info->ndims;
    d.data = (void *)data;
    for (unsigned i = 0; i < info->ndims && i < zdf_max_dims; i++) d.count[i] = info->count[i];
    const size_t ok = zdf_add_dataset(&zdf, &d);
    return zdf_close_file(&zdf) && ok;
}

EXPORT int zdf_open_part_file(t_zdf_file *zdf, t_zdf_part_info *info, const t_zdf_iteration *it, char const path[])
{
    char fn[1024];
    make_path(path);
    snprintf(fn, sizeof(fn), "%s/%s-%s-%06u.zdf", path, "particles", info->name, (unsigned)it->n);
    if (!zdf_open_file(zdf, fn, ZDF_CREATE)) {
        fprintf(stderr, "(*error*) Unable to open ZDF file, aborting.\n");
        return 0;
    }
    if (!zdf_add_string(zdf, "TYPE", "particles") || !zdf_add_part_info(zdf, info) ||
        !zdf_add_iteration(zdf, it)) {
        zdf_close_file(zdf);
        return 0;
    }
    return 1;
}

EXPORT int zdf_add_quant_part_file(t_zdf_file *zdf, const char *name, const float *data, const uint64_t np)
{
    t_zdf_dataset d;
    memset(&d, 0, sizeof(d));
    d.name = (char *)name;
    d.data_type = zdf_float32;
    d.ndims = 1;
    d.count[0] = np;
    d.data = (void *)data;
    return zdf_add_dataset(zdf, &d) ? 1 : 0;
}

/* ------------------------------------------------------------------------- */
/* background writer                                                         */
/* ------------------------------------------------------------------------- */
typedef struct zdf_job {
    int (*run)(void *arg);  /* writes one file; returns 1 on success */
    void *arg;
    struct zdf_job *next;
} zdf_job;

static pthread_mutex_t q_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t q_cv = PTHREAD_COND_INITIALIZER;    /* work queued */
static pthread_cond_t q_done = PTHREAD_COND_INITIALIZER;  /* queue drained */
static zdf_job *q_head = NULL, *q_tail = NULL;
static int q_busy = 0;      /* a job is being written */
static int q_failed = 0;    /* failures since the last flush */
static int q_started = 0;

static void *writer_main(void *unused)
{
    (void)unused;
    pthread_mutex_lock(&q_mu);
    for (;;) {
        while (!q_head) pthread_cond_wait(&q_cv, &q_mu);
        zdf_job *j = q_head;
        q_head = j->next;
        if (!q_head) q_tail = NULL;
        q_busy = 1;
        pthread_mutex_unlock(&q_mu);
        const int ok = j->run(j->arg);
        free(j);
        pthread_mutex_lock(&q_mu);
        if (!ok) q_failed++;
        q_busy = 0;
        if (!q_head) pthread_cond_broadcast(&q_done);
    }
    return NULL;
}

static void flush_at_exit(void) { zdf_flush(); }

/* queues run(arg) on the writer thread (FIFO); returns 0 if it could not
 * be queued, in which case it runs here and now */
int zdf_async_submit(int (*run)(void *), void *arg)
{
    zdf_job *j = (zdf_job *)malloc(sizeof(zdf_job));
    pthread_mutex_lock(&q_mu);
    if (!q_started) {
        pthread_t th;
        if (j && pthread_create(&th, NULL, writer_main, NULL) == 0) {
            pthread_detach(th);
            q_started = 1;
            atexit(flush_at_exit);
        }
    }
    if (!j || !q_started) {
        pthread_mutex_unlock(&q_mu);
        free(j);
        const int ok = run(arg);
        if (!ok) {
            pthread_mutex_lock(&q_mu);
            q_failed++;
            pthread_mutex_unlock(&q_mu);
        }
        return 0;
    }
    j->run = run;
    j->arg = arg;
    j->next = NULL;
    if (q_tail) q_tail->next = j;
    else q_head = j;
    q_tail = j;
    pthread_cond_signal(&q_cv);
    pthread_mutex_unlock(&q_mu);
    return 1;
}

EXPORT int zdf_flush(void)
{
    pthread_mutex_lock(&q_mu);
    while (q_head || q_busy) pthread_cond_wait(&q_done, &q_mu);
    const int failed = q_failed;
    q_failed = 0;
    pthread_mutex_unlock(&q_mu);
    return failed;
}
