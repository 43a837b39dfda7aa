/*
 * gpugrid_io.h -- dataset loaders of libgpugrid.so: the OSKAR binary
 * container of the visibility files (.vis) and the FITS cubes of the
 * W-kernels.  Host code, no GPU involved.
 *
 * These are the readers the reference's driver uses before it grids
 * (main.cpp:99-189 and :241-272 of the reference project):
 *
 *   oskar_binary_create / _free / _num_tags / _query / _read_block / _read /
 *   _read_int / _read_double   replace utils/binary/oskar_binary_create.h:56,
 *       oskar_binary_free.h, oskar_binary_query.h:45-110 and
 *       oskar_binary_read.h:60-152 (same names, arguments and int* status
 *       codes; opening for 'w' or 'a' is not provided and fails with
 *       OSKAR_ERR_BINARY_OPEN_FAIL; a file that fails to index returns NULL
 *       with the status set; payloads written big-endian are refused with
 *       OSKAR_ERR_BINARY_ENDIAN_MISMATCH);
 *   gg_vis_read_coords / gg_vis_scale_coords   replace read_coords and
 *       scale_coords (utils/read_vis.h:60-66, read_vis.c:31-73), renamed so
 *       that the library exports no unprefixed generic names;
 *   gg_read_kernel   replaces read_kernel (utils/read_kernel.h,
 *       read_kernel.c:36-118) without cfitsio: it returns a malloc'd cube
 *       [num_w_planes][conv_size_half][conv_size_half] in the requested
 *       precision and, when support is non-NULL, a calloc'd support table;
 *       the caller frees both with free().  On failure *status is non-zero,
 *       gg_last_error() says why, NULL is returned and *support is left
 *       NULL (nothing to free).
 */
#ifndef GPUGRID_IO_H_
#define GPUGRID_IO_H_

#include <stddef.h>

#include "gpugrid.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Data type codes of the container (utils/binary/oskar_binary_data_types.h). */
enum
{
    OSKAR_CHAR = 0x01,
    OSKAR_INT = 0x02,
    OSKAR_SINGLE = 0x04,
    OSKAR_DOUBLE = 0x08,
    OSKAR_COMPLEX = 0x20,
    OSKAR_MATRIX = 0x40,
    OSKAR_SINGLE_COMPLEX = OSKAR_SINGLE | OSKAR_COMPLEX,
    OSKAR_DOUBLE_COMPLEX = OSKAR_DOUBLE | OSKAR_COMPLEX,
    OSKAR_SINGLE_COMPLEX_MATRIX = OSKAR_SINGLE | OSKAR_COMPLEX | OSKAR_MATRIX,
    OSKAR_DOUBLE_COMPLEX_MATRIX = OSKAR_DOUBLE | OSKAR_COMPLEX | OSKAR_MATRIX
};

/* Tag groups of a visibility file (utils/binary/oskar_binary.h:69-70). */
enum
{
    OSKAR_TAG_GROUP_VIS_HEADER = 11,
    OSKAR_TAG_GROUP_VIS_BLOCK = 12
};

/* Header and block tags the reference's driver reads
 * (utils/read_vis.h:39-59). */
enum
{
    OSKAR_VIS_HEADER_TAG_NUM_TAGS_PER_BLOCK = 2,
    OSKAR_VIS_HEADER_TAG_AMP_TYPE = 5,
    OSKAR_VIS_HEADER_TAG_COORD_PRECISION = 6,
    OSKAR_VIS_HEADER_TAG_MAX_TIMES_PER_BLOCK = 7,
    OSKAR_VIS_HEADER_TAG_NUM_TIMES_TOTAL = 8,
    OSKAR_VIS_HEADER_TAG_MAX_CHANNELS_PER_BLOCK = 9,
    OSKAR_VIS_HEADER_TAG_NUM_CHANNELS_TOTAL = 10,
    OSKAR_VIS_HEADER_TAG_NUM_STATIONS = 11,
    OSKAR_VIS_HEADER_TAG_FREQ_START_HZ = 23
};
enum
{
    OSKAR_VIS_BLOCK_TAG_DIM_START_AND_SIZE = 1,
    OSKAR_VIS_BLOCK_TAG_CROSS_CORRELATIONS = 3,
    OSKAR_VIS_BLOCK_TAG_BASELINE_UU = 4,
    OSKAR_VIS_BLOCK_TAG_BASELINE_VV = 5,
    OSKAR_VIS_BLOCK_TAG_BASELINE_WW = 6
};

/* Status codes (utils/binary/oskar_binary.h:98-116). */
enum
{
    OSKAR_ERR_BINARY_OPEN_FAIL = -100,
    OSKAR_ERR_BINARY_SEEK_FAIL = -101,
    OSKAR_ERR_BINARY_READ_FAIL = -102,
    OSKAR_ERR_BINARY_WRITE_FAIL = -103,
    OSKAR_ERR_BINARY_NOT_OPEN_FOR_READ = -104,
    OSKAR_ERR_BINARY_NOT_OPEN_FOR_WRITE = -105,
    OSKAR_ERR_BINARY_FILE_INVALID = -106,
    OSKAR_ERR_BINARY_FORMAT_BAD = -107,
    OSKAR_ERR_BINARY_ENDIAN_MISMATCH = -108,
    OSKAR_ERR_BINARY_VERSION_UNKNOWN = -109,
    OSKAR_ERR_BINARY_TYPE_UNKNOWN = -110,
    OSKAR_ERR_BINARY_INT_UNKNOWN = -111,
    OSKAR_ERR_BINARY_FLOAT_UNKNOWN = -112,
    OSKAR_ERR_BINARY_DOUBLE_UNKNOWN = -113,
    OSKAR_ERR_BINARY_MEMORY_NOT_ALLOCATED = -114,
    OSKAR_ERR_BINARY_TAG_NOT_FOUND = -115,
    OSKAR_ERR_BINARY_TAG_TOO_LONG = -116,
    OSKAR_ERR_BINARY_TAG_OUT_OF_RANGE = -117,
    OSKAR_ERR_BINARY_CRC_FAIL = -118
};

typedef struct oskar_Binary oskar_Binary;

/* Opens `filename` for reading ('r') and indexes its chunks. */
GG_API oskar_Binary* oskar_binary_create(const char* filename, char mode,
        int* status);
GG_API void oskar_binary_free(oskar_Binary* handle);
GG_API int oskar_binary_num_tags(const oskar_Binary* handle);
/* Index of the first standard chunk with this type (0 = any), group, tag
 * and user index; -1 and OSKAR_ERR_BINARY_TAG_NOT_FOUND if none. */
GG_API int oskar_binary_query(const oskar_Binary* handle,
        unsigned char data_type, unsigned char id_group, unsigned char id_tag,
        int user_index, size_t* payload_size, int* status);
/* Copies chunk `chunk_index`'s payload to data (data_size bytes at least)
 * and checks its CRC-32C when the chunk carries one. */
GG_API void oskar_binary_read_block(oskar_Binary* handle, int chunk_index,
        size_t data_size, void* data, int* status);
GG_API void oskar_binary_read(oskar_Binary* handle, unsigned char data_type,
        unsigned char id_group, unsigned char id_tag, int user_index,
        size_t data_size, void* data, int* status);
GG_API void oskar_binary_read_int(oskar_Binary* handle,
        unsigned char id_group, unsigned char id_tag, int user_index,
        int* value, int* status);
GG_API void oskar_binary_read_double(oskar_Binary* handle,
        unsigned char id_group, unsigned char id_tag, int user_index,
        double* value, int* status);

/* Baseline coordinates (metres) of visibility block i_block. */
GG_API void gg_vis_read_coords(oskar_Binary* h, int i_block, int precision,
        size_t num_coords, void* uu, void* vv, void* ww, int* status);
/* Metres to wavelengths at freq_hz, in place. */
GG_API void gg_vis_scale_coords(double freq_hz, int precision,
        size_t num_coords, void* uu, void* vv, void* ww);

/* A W-kernel cube and its header keys from a FITS file. */
GG_API void* gg_read_kernel(const char* file_name, int precision,
        int* conv_size_half, int* num_w_planes, int** support,
        int* oversample, int* grid_size, double* cellsize_rad,
        double* w_scale, int* status);

#ifdef __cplusplus
}
#endif

#endif /* GPUGRID_IO_H_ */
