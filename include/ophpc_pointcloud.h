/*
 * C ABI over the ophPointCloud façade (include/ophPointCloud.h), for callers
 * that bind C rather than C++ (ctypes, cgo, JNI, N-API). One handle = one
 * ophPointCloud object; the functions map one to one onto its methods:
 *
 *   ophpc_pc_create / _release        new ophPointCloud() / release()
 *                                     (ophgen/src/ophPointCloud.cpp:51-62, Base.h:88-96)
 *   ophpc_pc_read_config              readConfig        (ophPointCloud.cpp:83-149)
 *   ophpc_pc_load_point_cloud         loadPointCloud    (ophPointCloud.cpp:73-76)
 *   ophpc_pc_set_point_cloud          setNumberOfPoints + setPointCloudModel (ophPointCloud.h:577-586)
 *   ophpc_pc_set_mode                 SetMode           (ophGen.h:529)
 *   ophpc_pc_set_viewing_window       setViewingWindow  (ophPointCloud.cpp:78-81)
 *   ophpc_pc_set_scale / _distance    setScale / setDistance (ophPointCloud.h:570-571)
 *   ophpc_pc_set_offset               Openholo::setOffset (Openholo.h:281)
 *   ophpc_pc_generate_hologram        generateHologram  (ophPointCloud.cpp:151-191)
 *   ophpc_pc_encoding                 encoding          (ophPointCloud.cpp:242-245)
 *   ophpc_pc_encoding_passband        encoding(flag, passband) (ophPointCloud.cpp:247-251)
 *   ophpc_pc_normalize                normalize         (ophGen.cpp:654-687)
 *   ophpc_pc_save                     save              (ophGen.cpp:689-769)
 *   ophpc_pc_save_ohc / _load_ohc     Openholo::saveAsOhc / loadAsOhc (Openholo.cpp:252-319)
 *   ophpc_pc_complex_field / _encoded / _normalized
 *                                     getComplexField()[ch] / getEncodedBuffer()[ch] /
 *                                     getNormalizedBuffer()[ch] (ophGen.h:117-124, Openholo.h:490)
 * Boolean results are 1 / 0. Buffers returned stay owned by the object and
 * valid until the next readConfig or release.
 */
#ifndef OPHPC_POINTCLOUD_H
#define OPHPC_POINTCLOUD_H

#include "ophpc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ophpc_pc ophpc_pc;

ophpc_pc* ophpc_pc_create(void);
void ophpc_pc_release(ophpc_pc* h);
int32_t ophpc_pc_read_config(ophpc_pc* h, const char* xml_path);
int64_t ophpc_pc_load_point_cloud(ophpc_pc* h, const char* ply_path);
void ophpc_pc_set_point_cloud(ophpc_pc* h, const ophpc_vertex* vertices, uint64_t n_points);
void ophpc_pc_set_mode(ophpc_pc* h, uint32_t mode);
void ophpc_pc_set_viewing_window(ophpc_pc* h, int32_t on);
void ophpc_pc_set_scale(ophpc_pc* h, double sx, double sy, double sz);
void ophpc_pc_set_distance(ophpc_pc* h, double distance);
void ophpc_pc_set_offset(ophpc_pc* h, int32_t ox, int32_t oy);
double ophpc_pc_generate_hologram(ophpc_pc* h, uint32_t diff_flag);
void ophpc_pc_encoding(ophpc_pc* h, uint32_t encode_flag);
/* encoding(flag, passband) (ophPointCloud.cpp:247-251): OPHPC_ENCODE_SSB,
 * OPHPC_ENCODE_OFFSSB with an OPHPC_SSB_* passband. */
void ophpc_pc_encoding_passband(ophpc_pc* h, uint32_t encode_flag, uint32_t passband);
void ophpc_pc_normalize(ophpc_pc* h);
int32_t ophpc_pc_save(ophpc_pc* h, const char* path, uint8_t bits_per_pixel);
int32_t ophpc_pc_save_ohc(ophpc_pc* h, const char* path);
int32_t ophpc_pc_load_ohc(ophpc_pc* h, const char* path);
int32_t ophpc_pc_get_config(ophpc_pc* h, ophpc_config* out);
uint64_t ophpc_pc_number_of_points(ophpc_pc* h);
const ophpc_vertex* ophpc_pc_point_cloud(ophpc_pc* h);
const double* ophpc_pc_complex_field(ophpc_pc* h, uint32_t channel);
const double* ophpc_pc_encoded(ophpc_pc* h, uint32_t channel);
const uint8_t* ophpc_pc_normalized(ophpc_pc* h, uint32_t channel);
const char* ophpc_pc_last_error(ophpc_pc* h);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_POINTCLOUD_H */
