/*
 * ophpc I/O — config, point-cloud and image files of the point-cloud path
 * (C ABI; host-only, no GPU needed).
 *
 *   ophpc_read_config  replaces ophGen::readConfig + ophPointCloud::readConfig
 *                      (ophgen/src/ophGen.cpp:221-358,
 *                       ophgen/src/ophPointCloud.cpp:83-149)
 *   ophpc_load_ply     replaces PLYparser::loadPLY
 *                      (Openholo/src/PLYparser.cpp:142-449)
 *   ophpc_save_bmp     replaces Openholo::saveAsImg
 *                      (Openholo/src/Openholo.cpp:135-251)
 */
#ifndef OPHPC_IO_H
#define OPHPC_IO_H

#include "ophpc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ImageConfig (Openholo/src/Openholo.h:122-131) + the optional keys of the
 * common config that the point-cloud path reads but does not use. */
typedef struct ophpc_image_config {
    int32_t rotate;          /* IMG_Rotation, default 0 */
    int32_t merge;           /* IMG_Merge, default 0 */
    int32_t flip;            /* IMG_Flip: 0 none, 1 vertical, 2 horizontal, 3 both */
    int32_t double_precision;/* DoublePrecision, default 1 */
    double shift[3];         /* ShiftX/Y/Z, default 0 */
    int32_t random_phase;    /* RandomPhase, default 0 */
    int32_t num_of_stream;   /* NumOfStream, default 1 */
} ophpc_image_config;

/* Parses the flat <PointCloud> XML config. Fills cfg (pixel_number,
 * pixel_pitch, n_channels, wave_length, scale, distance, field_length; offset
 * and viewing_window are left 0) and, if img is non-NULL, the optional keys.
 * Returns OPHPC_ERROR_IO when the file cannot be read or is not ".xml",
 * OPHPC_ERROR_CONFIG when a required key is missing or malformed (cfg still
 * holds every key that was read, as the reference leaves them), else
 * OPHPC_SUCCESS. More than OPHPC_MAX_CHANNELS wavelengths is a config error.
 * Keys parse like tinyxml2's Query*Text: leading whitespace skipped, a
 * numeric prefix accepted, booleans as integers or true/false. */
ophpc_status ophpc_read_config(const char* xml_path, ophpc_config* cfg, ophpc_image_config* img);

/* Loads a PLY point cloud (ASCII, binary_little_endian or
 * binary_big_endian) into 56-byte vertex records. With out == NULL only the
 * header is read and its vertex count returned (the data are checked by the
 * loading call). With capacity >= the count the records are decoded
 * straight into out (which may be page-locked memory); otherwise the first
 * `capacity` records are copied. Returns the vertex count, or -1 on error
 * (unreadable file, malformed header, truncated data). Colours are
 * (double)(c / 255.f) from red/green/blue (or diffuse_*); a file without a
 * `color` element with a `channel` property gets 0.5 in every channel, as
 * the reference does. */
int64_t ophpc_load_ply(const char* path, ophpc_vertex* out, uint64_t capacity);

/* Writes an uncompressed BMP: 8 bits per pixel with a 256-entry grey
 * palette, or 24 bits per pixel (BGR) from an interleaved buffer. Rows are
 * written in buffer order, each padded to 4 bytes. flip: 0 none,
 * 1 vertical, 2 horizontal, 3 both; rotate != 0 rotates by 180 degrees. */
ophpc_status ophpc_save_bmp(const char* path, const uint8_t* pixels, int32_t width, int32_t height,
                            int32_t bits_per_pixel, int32_t flip, int32_t rotate);

/* Openholo complex-field file (.ohc; Openholo/src/ImgCodecDefine.h:53-210,
 * Openholo/src/ImgCodecOhc.cpp): writes the field as the reference's
 * Openholo::saveAsOhc does (Openholo/src/Openholo.cpp:252-279) — version
 * 3.0, real/imaginary float64, one plane per channel, metres — byte for
 * byte. field: [n_channels][pnY][pnX][re, im] doubles. ".ohc" is appended
 * when the name does not end in it. */
ophpc_status ophpc_save_ohc(const char* path, const double* field, int32_t pnx, int32_t pny, double ppx,
                            double ppy, uint32_t n_channels, const double* wavelengths);

/* Reads a .ohc (Openholo::loadAsOhc, Openholo/src/Openholo.cpp:280-319;
 * ImgDecoderOhc::decodeFieldData, Openholo/src/ImgCodecOhc.cpp:434-600):
 * real/imaginary float32 or float64, one plane per channel or channels
 * interleaved per pixel; pitch and wavelengths returned as stored, as the
 * reference does. Amplitude/phase files are converted to real/imaginary
 * (the reference leaves its complex field zero for them). Fills the shape
 * (any pointer may be NULL) and, when field is non-NULL and
 * capacity_doubles suffices (2 * n_channels * pnX * pnY), the field in the
 * layout of ophpc_save_ohc. More than OPHPC_MAX_CHANNELS wavelengths,
 * linked-file storage or amplitude-only / phase-only coding is
 * OPHPC_ERROR_UNSUPPORTED. */
ophpc_status ophpc_load_ohc(const char* path, int32_t* pnx, int32_t* pny, double* ppx, double* ppy,
                            uint32_t* n_channels, double* wavelengths, double* field, uint64_t capacity_doubles);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_IO_H */
