/*
 * zdf.h -- ZDF diagnostic files (the writing half of ZPIC's em2d/zdf.h).
 *
 * The structs, enums and function signatures are those of the reference
 * interface (em2d/zdf.h:36-420), so that decks and diagnostics written
 * against it compile unchanged; the implementation (zdf_io.c) is this
 * library's own.  A file is the 4-byte magic "ZDF1" followed by records:
 * a uint32 id/version, the record name as a string (uint32 length, bytes,
 * zero padding to a multiple of 4), a uint64 payload length, then the
 * payload.  Every number is little endian.
 *
 * Beyond the reference: zdf_flush() waits for the report files that
 * libzpic_em2d writes on its background thread (see simulation.h).
 */
#ifndef ZPIC_EM2D_ZDF_H
#define ZPIC_EM2D_ZDF_H

#include <stdint.h>
#include <stdio.h>

#define BYTES_PER_ZDF_UNIT (4)
#define ZDF_MAGIC_LENGTH BYTES_PER_ZDF_UNIT
#define zdf_max_dims 3

enum zdf_data_type {
    zdf_null,
    zdf_int8,
    zdf_uint8,
    zdf_int16,
    zdf_uint16,
    zdf_int32,
    zdf_uint32,
    zdf_int64,
    zdf_uint64,
    zdf_float32,
    zdf_float64
};

enum zdf_file_access_mode { ZDF_CREATE, ZDF_READ, ZDF_UPDATE };

typedef struct ZDF_File {
    FILE *fp;
    enum zdf_file_access_mode mode;
    uint32_t ndatasets;
} t_zdf_file;

typedef struct ZDF_Dataset {
    char *name;
    enum zdf_data_type data_type;
    uint32_t ndims;
    uint64_t count[zdf_max_dims];
    void *data;
    uint64_t id;
    uint64_t offset;
} t_zdf_dataset;

typedef struct ZDF_Chunk {
    uint64_t count[zdf_max_dims];
    uint64_t start[zdf_max_dims];
    uint64_t stride[zdf_max_dims];
    void *data;
} t_zdf_chunk;

enum zdf_axis_type { zdf_linear, zdf_log10, zdf_log2 };

typedef struct ZDF_GridAxis {
    char *name;
    enum zdf_axis_type type;
    double min;
    double max;
    char *label;
    char *units;
} t_zdf_grid_axis;

typedef struct ZDF_GridInfo {
    char *name;
    uint32_t ndims;
    uint64_t count[zdf_max_dims];
    char *label;
    char *units;
    t_zdf_grid_axis *axis;
} t_zdf_grid_info;

typedef struct ZDF_Iteration {
    char *name;
    int32_t n;
    double t;
    char *time_units;
} t_zdf_iteration;

typedef struct ZDF_PartInfo {
    char *name;
    char *label;
    uint64_t np;
    uint32_t nquants;
    char **quants;
    char **qlabels;
    char **qunits;
} t_zdf_part_info;

typedef struct ZDF_TrackInfo {
    char *name;
    char *label;
    uint32_t ntracks;
    uint32_t ndump;
    uint32_t niter;
    uint32_t nquants;
    char **quants;
    char **qlabels;
    char **qunits;
} t_zdf_track_info;

/* low level: every call returns the bytes written (0 on error), except
 * open / close, which return 1 on success and 0 on error */
size_t zdf_sizeof(enum zdf_data_type data_type);
int zdf_open_file(t_zdf_file *zdf, const char *filename, enum zdf_file_access_mode mode);
int zdf_close_file(t_zdf_file *zdf);
size_t zdf_vector_write(t_zdf_file *zdf, const void *data, enum zdf_data_type data_type, size_t len);
size_t zdf_add_string(t_zdf_file *zdf, const char *name, const char *str);
size_t zdf_add_int32(t_zdf_file *zdf, const char *name, const int32_t value);
size_t zdf_add_double(t_zdf_file *zdf, const char *name, const double value);
size_t zdf_add_iteration(t_zdf_file *zdf, const t_zdf_iteration *iter);
size_t zdf_add_grid_info(t_zdf_file *zdf, const t_zdf_grid_info *grid);
size_t zdf_add_part_info(t_zdf_file *zdf, const t_zdf_part_info *part);
size_t zdf_add_track_info(t_zdf_file *zdf, const t_zdf_track_info *tracks);
size_t zdf_add_dataset(t_zdf_file *zdf, t_zdf_dataset *dataset);
size_t zdf_start_cdset(t_zdf_file *zdf, t_zdf_dataset *dataset);
size_t size_zdf_chunk_header(const t_zdf_dataset *dataset);
size_t zdf_write_chunk_header(t_zdf_file *zdf, t_zdf_dataset *dataset, t_zdf_chunk *chunk);
size_t zdf_write_cdset(t_zdf_file *zdf, t_zdf_dataset *dataset, t_zdf_chunk *chunk);
size_t zdf_end_cdset(t_zdf_file *zdf, t_zdf_dataset *dataset);

/* high level: "<path>/<name>-<n:06>.zdf" grid files and
 * "<path>/particles-<name>-<n:06>.zdf" particle files; the path is created
 * as needed.  Return 1 on success, 0 on error. */
int zdf_open_grid_file(t_zdf_file *file, const t_zdf_grid_info *info, const t_zdf_iteration *iteration,
                       char const path[]);
int zdf_save_grid(const void *data, enum zdf_data_type data_type, const t_zdf_grid_info *info,
                  const t_zdf_iteration *iteration, char const path[]);
int zdf_open_part_file(t_zdf_file *file, t_zdf_part_info *info, const t_zdf_iteration *iteration,
                       char const path[]);
int zdf_add_quant_part_file(t_zdf_file *zdf, const char *name, const float *data, const uint64_t np);

/* waits until every report file queued so far is on disk; returns the
 * number of files that could not be written */
int zdf_flush(void);

#endif
