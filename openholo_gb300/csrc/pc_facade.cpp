// ophPointCloud façade (include/ophPointCloud.h) and its C ABI
// (include/ophpc_pointcloud.h).
//
// Mirrors the reference object's state and call sequence
// (ophgen/src/ophPointCloud.cpp, ophgen/src/ophGen.cpp:146-219,654-849):
// host buffers complex_H / m_lpEncoded / m_lpNormalized per channel, filled
// by generateHologram / encoding / normalize; the arithmetic runs in
// libophpc's kernels. Every call that reads a host buffer uploads it first,
// so a caller that edits getComplexField() or getEncodedBuffer() between
// calls sees the same result as with the reference.
#include "ophPointCloud.h"
#include "ophpc_pointcloud.h"

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

static_assert(sizeof(Complex<Real>) == 2 * sizeof(Real) && std::is_trivially_copyable<Complex<Real>>::value,
              "complex_H elements are plain {re, im} pairs");

#define OPH_LOG(...) std::printf(__VA_ARGS__)

namespace {
constexpr double kPi = 3.14159265358979323846;

// The per-channel host buffers are page-locked when the CUDA runtime can
// provide it, so that the uploads and downloads around every call run at
// the link's speed; without a device (readConfig works without one) they are
// ordinary heap memory. Either way they start zeroed.
void* host_alloc(size_t bytes, bool pinned) {
    void* p = nullptr;
    if (pinned) {
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    } else {
        p = ::operator new(bytes);
    }
    std::memset(p, 0, bytes);
    return p;
}

void host_free(void* p, bool pinned) {
    if (!p) return;
    if (pinned) cudaFreeHost(p);
    else ::operator delete(p);
}

// The point records: page-locked when the runtime can provide it (their
// upload in generateHologram then runs at the link's speed), else on the heap.
Vertex* vertices_alloc(size_t n, bool& pinned) {
    void* p = nullptr;
    pinned = cudaHostAlloc(&p, sizeof(Vertex) * (n ? n : 1), cudaHostAllocDefault) == cudaSuccess;
    if (!pinned) {
        cudaGetLastError();
        p = ::operator new(sizeof(Vertex) * (n ? n : 1));
    }
    return static_cast<Vertex*>(p);
}

void vertices_free(Vertex* p, bool pinned) { host_free(p, pinned); }

// memcpy in one part below 4 MiB, two threads' parts from 4 MiB and four
// from 8 MiB (one core's copy rate is a fraction of the memory system's)
void copy_parallel(void* dst, const void* src, size_t bytes) {
    constexpr size_t kChunkMin = (size_t)2 << 20;
    const size_t parts = bytes >= 4 * kChunkMin ? 4 : bytes >= 2 * kChunkMin ? 2 : 1;
    if (parts == 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t per = (bytes / parts + 63) / 64 * 64;
    std::vector<std::thread> ts;
    for (size_t i = 1; i < parts; ++i) {
        const size_t off = i * per;
        if (off >= bytes) break;
        const size_t len = off + per <= bytes ? per : bytes - off;
        auto part = [=] { std::memcpy((char*)dst + off, (const char*)src + off, len); };
        try {
            ts.emplace_back(part);
        } catch (...) {   // no thread to be had: this one copies the part
            part();
        }
    }
    std::memcpy(dst, src, per < bytes ? per : bytes);
    for (auto& t : ts) t.join();
}
}  // namespace

ophPointCloud::ophPointCloud(void) { context_.wave_length = wave_length_; }

ophPointCloud::ophPointCloud(const char* pc_file, const char* cfg_file) : ophPointCloud() {
    if (loadPointCloud(pc_file) == -1) OPH_LOG("<FAILED> Load point cloud data file('%s')", pc_file);
    if (!readConfig(cfg_file)) OPH_LOG("<FAILED> Load config specification data file('%s')", cfg_file);
}

ophPointCloud::~ophPointCloud(void) {
    freeBuffers();
    vertices_free(vertices_, vertices_pinned_);
    vertices_ = nullptr;
    if (d_vertices_) cudaFree(d_vertices_);
    if (d_field_) cudaFree(d_field_);
    if (d_encoded_) cudaFree(d_encoded_);
    if (d_codes_) cudaFree(d_codes_);
    for (void* st : streams_)
        if (st) cudaStreamDestroy((cudaStream_t)st);
    if (gpu_) ophpc_destroy(gpu_);
}

void ophPointCloud::release(void) { delete this; }

void ophPointCloud::freeBuffers() {
    for (uint c = 0; c < n_old_channels_; ++c) {
        if (complex_H_) host_free(complex_H_[c], host_pinned_);
        if (encoded_) host_free(encoded_[c], host_pinned_);
        if (normalized_) host_free(normalized_[c], host_pinned_);
    }
    delete[] complex_H_;
    delete[] encoded_;
    delete[] normalized_;
    complex_H_ = nullptr;
    encoded_ = nullptr;
    normalized_ = nullptr;
    n_old_channels_ = 0;
    buffer_pixels_ = 0;
}

bool ophPointCloud::initialize() {
    freeBuffers();
    const uint nch = context_.waveNum;
    const long long n = (long long)context_.pixel_number[_X] * context_.pixel_number[_Y];
    if (nch < 1 || nch > OPHPC_MAX_CHANNELS || n <= 0) return false;
    complex_H_ = new Complex<Real>*[nch]();
    encoded_ = new Real*[nch]();
    normalized_ = new uchar*[nch]();
    n_old_channels_ = nch;
    // page-locked if every buffer can be, else all on the heap
    for (int attempt = 0; attempt < 2; ++attempt) {
        host_pinned_ = attempt == 0;
        bool ok = true;
        for (uint c = 0; c < nch && ok; ++c) {
            // Complex<Real> is a pair of doubles with no state beyond it: a
            // zeroed buffer holds value-initialised elements
            complex_H_[c] = static_cast<Complex<Real>*>(host_alloc(sizeof(Complex<Real>) * (size_t)n, host_pinned_));
            encoded_[c] = static_cast<Real*>(host_alloc(sizeof(Real) * (size_t)n, host_pinned_));
            normalized_[c] = static_cast<uchar*>(host_alloc((size_t)n, host_pinned_));
            ok = complex_H_[c] && encoded_[c] && normalized_[c];
        }
        if (ok) break;
        for (uint c = 0; c < nch; ++c) {
            host_free(complex_H_[c], host_pinned_);
            host_free(encoded_[c], host_pinned_);
            host_free(normalized_[c], host_pinned_);
            complex_H_[c] = nullptr;
            encoded_[c] = nullptr;
            normalized_[c] = nullptr;
        }
    }
    buffer_pixels_ = n;
    return true;
}

void ophPointCloud::setPixelNumber(int nx, int ny) {
    context_.pixel_number[_X] = nx;
    context_.pixel_number[_Y] = ny;
    context_.ss[_X] = nx * context_.pixel_pitch[_X];
    context_.ss[_Y] = ny * context_.pixel_pitch[_Y];
    initialize();
}

void ophPointCloud::setPixelPitch(Real px, Real py) {
    context_.pixel_pitch[_X] = px;
    context_.pixel_pitch[_Y] = py;
    context_.ss[_X] = context_.pixel_number[_X] * px;
    context_.ss[_Y] = context_.pixel_number[_Y] * py;
}

void ophPointCloud::setWaveNum(uint n) {
    context_.waveNum = n > OPHPC_MAX_CHANNELS ? OPHPC_MAX_CHANNELS : n;
    initialize();
}

void ophPointCloud::setWaveLength(Real w, uint idx) {
    if (idx < OPHPC_MAX_CHANNELS) wave_length_[idx] = w;
}

bool ophPointCloud::readConfig(const char* cfg_file) {
    ophpc_config c;
    ophpc_image_config img;
    std::memset(&img, 0, sizeof(img));
    const ophpc_status st = ophpc_read_config(cfg_file, &c, &img);
    if (st == OPHPC_ERROR_IO || st == OPHPC_ERROR_INVALID_ARGUMENT) {
        OPH_LOG("<FAILED> Loading file\n");
        last_error_ = "cannot read config file";
        return false;
    }
    context_.waveNum = c.n_channels;
    for (uint i = 0; i < OPHPC_MAX_CHANNELS; ++i) wave_length_[i] = c.wave_length[i];
    context_.pixel_number[_X] = c.pixel_number[0];
    context_.pixel_number[_Y] = c.pixel_number[1];
    context_.pixel_pitch[_X] = c.pixel_pitch[0];
    context_.pixel_pitch[_Y] = c.pixel_pitch[1];
    context_.ss[_X] = context_.pixel_number[_X] * context_.pixel_pitch[_X];
    context_.ss[_Y] = context_.pixel_number[_Y] * context_.pixel_pitch[_Y];
    context_.bUseDP = img.double_precision != 0;
    for (int i = 0; i < 3; ++i) context_.shift[i] = img.shift[i];
    img_ = img;
    field_length_ = c.field_length;
    scale_[0] = c.scale[0];
    scale_[1] = c.scale[1];
    scale_[2] = c.scale[2];
    distance_ = c.distance;
    if (st != OPHPC_SUCCESS) {
        last_error_ = "config key missing or malformed";
        // the reference initialises only once the common keys were read
        if (c.pixel_number[0] > 0 && c.pixel_number[1] > 0 && c.pixel_pitch[0] > 0 && c.pixel_pitch[1] > 0)
            initialize();
        return false;
    }
    if (!initialize()) {
        last_error_ = "invalid pixel number or channel count";
        return false;
    }
    return true;
}

int ophPointCloud::loadPointCloud(const char* pc_file) {
    const int64_t n = ophpc_load_ply(pc_file, nullptr, 0);
    if (n < 0) {
        OPH_LOG("<FAILED> Loading ply file.\n");
        last_error_ = "cannot load point cloud";
        return -1;
    }
    bool pinned = false;
    Vertex* v = vertices_alloc((size_t)n, pinned);
    if (ophpc_load_ply(pc_file, reinterpret_cast<ophpc_vertex*>(v), (uint64_t)n) != n) {
        vertices_free(v, pinned);
        OPH_LOG("<FAILED> Loading ply file.\n");
        last_error_ = "cannot load point cloud";
        return -1;
    }
    vertices_free(vertices_, vertices_pinned_);
    vertices_ = v;
    vertices_pinned_ = pinned;
    vertices_cap_ = (ulonglong)n;
    n_points_ = (ulonglong)n;
    return (int)n;
}

void ophPointCloud::setPointCloudModel(Vertex* vertex) {
    if (n_points_ < 1 || !vertex) return;
    if (vertices_ != vertex) {   // the copy (ophPointCloud.h:577-586); its buffer is reused at the same size
        if (!vertices_ || vertices_cap_ != n_points_) {
            vertices_free(vertices_, vertices_pinned_);
            vertices_ = vertices_alloc((size_t)n_points_, vertices_pinned_);
            vertices_cap_ = n_points_;
        }
        copy_parallel(vertices_, vertex, sizeof(Vertex) * n_points_);
    }
}

void ophPointCloud::fillConfig(ophpc_config* c) const {
    std::memset(c, 0, sizeof(*c));
    c->pixel_number[0] = context_.pixel_number[_X];
    c->pixel_number[1] = context_.pixel_number[_Y];
    c->offset[0] = context_.offset[_X];
    c->offset[1] = context_.offset[_Y];
    c->pixel_pitch[0] = context_.pixel_pitch[_X];
    c->pixel_pitch[1] = context_.pixel_pitch[_Y];
    for (int i = 0; i < 3; ++i) c->scale[i] = scale_[i];
    c->distance = distance_;
    c->field_length = field_length_;
    c->viewing_window = viewing_window_ ? 1 : 0;
    c->n_channels = context_.waveNum;
    for (uint i = 0; i < OPHPC_MAX_CHANNELS; ++i) c->wave_length[i] = wave_length_[i];
}

bool ophPointCloud::ensureGpu() {
    if (gpu_) return true;
    const ophpc_status st = ophpc_create(0, &gpu_);
    if (st != OPHPC_SUCCESS) {
        gpu_ = nullptr;
        last_error_ = std::string("no GPU context: ") + ophpc_status_string(st);
        OPH_LOG("<FAILED> %s\n", last_error_.c_str());
        return false;
    }
    return true;
}

bool ophPointCloud::ensureDevice(size_t bv, size_t bf, size_t be, size_t bc) {
    auto grow = [&](void** p, size_t* cap, size_t want) {
        if (want <= *cap) return true;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        if (cudaMalloc(p, want) != cudaSuccess) {
            cudaGetLastError();
            *p = nullptr;
            return false;
        }
        *cap = want;
        return true;
    };
    if (!grow(&d_vertices_, &cap_v_, bv) || !grow(&d_field_, &cap_f_, bf) || !grow(&d_encoded_, &cap_e_, be) ||
        !grow(&d_codes_, &cap_c_, bc)) {
        last_error_ = "device allocation failed";
        return false;
    }
    return true;
}

bool ophPointCloud::ensureStreams() {
    for (uint ch = 0; ch < OPHPC_MAX_CHANNELS; ++ch) {
        if (streams_[ch]) continue;
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            last_error_ = "stream creation failed";
            return false;
        }
        streams_[ch] = st;
    }
    return true;
}

Real ophPointCloud::generateHologram(uint diff_flag) {
    const auto begin = std::chrono::steady_clock::now();
    if (diff_flag != PC_DIFF_RS && diff_flag != PC_DIFF_FRESNEL) {
        OPH_LOG("<FAILED> Wrong parameters.");
        return 0.0;
    }
    if (!complex_H_) {
        last_error_ = "readConfig must succeed before generateHologram";
        return 0.0;
    }
    // resetBuffer (ophGen.cpp:801-814), on a helper thread while the GPU
    // generates: the buffers are back to zero before this call returns
    struct Joiner {
        std::thread t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } reset;
    {
        Real** enc = encoded_;
        uchar** nrm = normalized_;
        const uint nch_reset = context_.waveNum;
        const size_t px = (size_t)buffer_pixels_;
        auto clear = [enc, nrm, nch_reset, px] {
            for (uint c = 0; c < nch_reset; ++c) {
                std::memset(enc[c], 0, sizeof(Real) * px);
                std::memset(nrm[c], 0, px);
            }
        };
        try {
            reset.t = std::thread(clear);
        } catch (...) {   // no thread to be had: clear them here
            clear();
        }
    }
    encoded_valid_ = false;
    if (!ensureGpu()) return 0.0;
    if (n_points_ > 0 && !vertices_) {
        last_error_ = "no point cloud";
        return 0.0;
    }
    ophpc_config c;
    fillConfig(&c);
    const size_t plane = (size_t)buffer_pixels_;
    const uint nch = context_.waveNum;
    if (!ensureDevice(sizeof(Vertex) * (n_points_ ? n_points_ : 1), sizeof(double) * 2 * plane * nch,
                      sizeof(double) * plane * nch, plane * nch))
        return 0.0;
    if (n_points_ && cudaMemcpy(d_vertices_, vertices_, sizeof(Vertex) * n_points_, cudaMemcpyHostToDevice) != cudaSuccess) {
        last_error_ = "vertex upload failed";
        return 0.0;
    }
    const ophpc_status st = ophpc_generate(gpu_, &c, reinterpret_cast<const ophpc_vertex*>(d_vertices_), n_points_,
                                           diff_flag, mode_, (double*)d_field_, nullptr);
    if (st != OPHPC_SUCCESS) {
        last_error_ = std::string("generate: ") + ophpc_last_error(gpu_);
        return 0.0;
    }
    // the channels' downloads queued behind the generate, one wait
    bool ok = true;
    for (uint ch = 0; ch < nch && ok; ++ch)
        ok = cudaMemcpyAsync(complex_H_[ch], (double*)d_field_ + 2 * plane * ch, sizeof(double) * 2 * plane,
                             cudaMemcpyDeviceToHost, nullptr) == cudaSuccess;
    if (cudaStreamSynchronize(nullptr) != cudaSuccess || !ok) {
        cudaGetLastError();
        last_error_ = "field download failed";
        return 0.0;
    }
    context_.k = (2 * kPi) / wave_length_[nch - 1];
    progress_ = 0;
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - begin).count();
}

void ophPointCloud::encoding(unsigned int flag) {
    if (flag > ENCODE_TWOPHASE) {
        OPH_LOG("<FAILED> WRONG PARAMETERS.\n");
        return;
    }
    if (!complex_H_ || !ensureGpu()) return;
    const size_t plane = (size_t)buffer_pixels_;
    const uint nch = context_.waveNum;
    if (!ensureDevice(cap_v_ ? cap_v_ : 1, sizeof(double) * 2 * plane * nch, sizeof(double) * plane * nch, plane * nch))
        return;
    // Every encoder works on one channel at a time (the normalising ones by
    // the channel's own largest magnitude), so the channels run as a
    // pipeline, one stream each: the upload of one overlaps the encoding and
    // the download of the one before.
    if (!ensureStreams()) return;
    cudaDeviceSynchronize();   // earlier work on the field buffers (legacy stream) is done
    bool ok = true;
    std::string err;
    for (uint ch = 0; ch < nch && ok; ++ch) {
        cudaStream_t st = (cudaStream_t)streams_[ch];
        double* df = (double*)d_field_ + 2 * plane * ch;
        double* de = (double*)d_encoded_ + plane * ch;
        ok = cudaMemcpyAsync(df, complex_H_[ch], sizeof(double) * 2 * plane, cudaMemcpyHostToDevice, st) ==
             cudaSuccess;
        // Burckhardt and TwoPhase leave some entries of m_lpEncoded as they were
        if (ok && (flag == ENCODE_BURCKHARDT || flag == ENCODE_TWOPHASE))
            ok = cudaMemcpyAsync(de, encoded_[ch], sizeof(double) * plane, cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (ok && ophpc_encode(gpu_, df, 1, plane, flag, de, nullptr, st) != OPHPC_SUCCESS) {
            err = std::string("encode: ") + ophpc_last_error(gpu_);
            ok = false;
        }
        if (ok) ok = cudaMemcpyAsync(encoded_[ch], de, sizeof(double) * plane, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    }
    for (uint ch = 0; ch < nch; ++ch)
        if (cudaStreamSynchronize((cudaStream_t)streams_[ch]) != cudaSuccess) ok = false;
    if (!ok) {
        cudaGetLastError();
        last_error_ = err.empty() ? std::string("encode copies failed") : err;
        return;
    }
    encoded_valid_ = true;
}

void ophPointCloud::encodeSideband(unsigned int flag, unsigned int passband, Real shift_x, Real shift_y) {
    if (!complex_H_ || !ensureGpu()) return;
    const size_t plane = (size_t)buffer_pixels_;
    const uint nch = context_.waveNum;
    if (!ensureDevice(cap_v_ ? cap_v_ : 1, sizeof(double) * 2 * plane * nch, sizeof(double) * plane * nch, plane * nch))
        return;
    context_.ss[_X] = context_.pixel_number[_X] * context_.pixel_pitch[_X];
    context_.ss[_Y] = context_.pixel_number[_Y] * context_.pixel_pitch[_Y];
    // uploads, the transforms and downloads queued on the legacy stream, one wait
    bool ok = true;
    std::string err;
    for (uint ch = 0; ch < nch && ok; ++ch)
        ok = cudaMemcpyAsync((double*)d_field_ + 2 * plane * ch, complex_H_[ch], sizeof(double) * 2 * plane,
                             cudaMemcpyHostToDevice, nullptr) == cudaSuccess;
    if (ok && ophpc_encode_ssb(gpu_, (const double*)d_field_, nch, context_.pixel_number[_X],
                               context_.pixel_number[_Y], context_.pixel_pitch[_X], context_.pixel_pitch[_Y], flag,
                               passband, shift_x, shift_y, (double*)d_encoded_, nullptr, nullptr) != OPHPC_SUCCESS) {
        err = std::string("encode: ") + ophpc_last_error(gpu_);
        ok = false;
    }
    for (uint ch = 0; ch < nch && ok; ++ch)
        ok = cudaMemcpyAsync(encoded_[ch], (double*)d_encoded_ + plane * ch, sizeof(double) * plane,
                             cudaMemcpyDeviceToHost, nullptr) == cudaSuccess;
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) ok = false;
    if (!ok) {
        cudaGetLastError();
        last_error_ = err.empty() ? std::string("encode copies failed") : err;
        OPH_LOG("<FAILED> %s\n", last_error_.c_str());
        return;
    }
    encoded_valid_ = true;
}

void ophPointCloud::encoding(unsigned int flag, unsigned int passband) {
    if (flag == ENCODE_SSB) encodeHologram();
    else if (flag == ENCODE_OFFSSB) encodeSideband(OPHPC_ENCODE_OFFSSB, passband, 0.0, 0.0);
}

void ophPointCloud::encodeHologram(const vec2 band_limit, const vec2 spectrum_shift) {
    (void)band_limit;
    if (!complex_H_) {
        OPH_LOG("<FAILED> Not found diffracted data.");
        return;
    }
    encodeSideband(OPHPC_ENCODE_SSB, 0, spectrum_shift[_X], spectrum_shift[_Y]);
}

void ophPointCloud::normalize(void) {
    if (!encoded_ || !ensureGpu()) return;
    const size_t plane = (size_t)buffer_pixels_;
    const uint nch = context_.waveNum;
    if (!ensureDevice(cap_v_ ? cap_v_ : 1, cap_f_ ? cap_f_ : 1, sizeof(double) * plane * nch, plane * nch)) return;
    if (!ensureStreams()) return;
    cudaDeviceSynchronize();   // earlier work on the buffers (legacy stream) is done
    // uploads, min/max and codes, downloads queued on one stream, one wait
    cudaStream_t st = (cudaStream_t)streams_[0];
    bool ok = true;
    std::string err;
    for (uint ch = 0; ch < nch && ok; ++ch)
        ok = cudaMemcpyAsync((double*)d_encoded_ + plane * ch, encoded_[ch], sizeof(double) * plane,
                             cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ok && ophpc_normalize(gpu_, (const double*)d_encoded_, nch, plane, (uint8_t*)d_codes_, st) != OPHPC_SUCCESS) {
        err = std::string("normalize: ") + ophpc_last_error(gpu_);
        ok = false;
    }
    for (uint ch = 0; ch < nch && ok; ++ch)
        ok = cudaMemcpyAsync(normalized_[ch], (uint8_t*)d_codes_ + plane * ch, plane, cudaMemcpyDeviceToHost, st) ==
             cudaSuccess;
    if (cudaStreamSynchronize(st) != cudaSuccess) ok = false;
    if (!ok) {
        cudaGetLastError();
        last_error_ = err.empty() ? std::string("normalize copies failed") : err;
    }
}

bool ophPointCloud::save(const char* fname, uint8_t bitsperpixel, uchar* src, uint px, uint py) {
    if (fname == nullptr) return false;
    int w = (int)px, h = (int)py;
    if (px == 0 && py == 0) {
        w = context_.pixel_number[_X];
        h = context_.pixel_number[_Y];
    }
    // ophGen::save (ophgen/src/ophGen.cpp:689-769): '\\' -> '/', ".bmp"
    // appended when the path has no '.'
    std::string file = fname;
    for (auto& ch : file)
        if (ch == '\\') ch = '/';
    const size_t slash = file.find_last_of('/');
    const std::string dir = slash == std::string::npos ? "" : file.substr(0, slash + 1);
    std::string name = slash == std::string::npos ? file : file.substr(slash + 1);
    if (file.rfind('.') == std::string::npos) name += ".bmp";
    const std::string full = dir + name;
    if (src) return ophpc_save_bmp(full.c_str(), src, w, h, bitsperpixel, img_.flip, img_.rotate) == OPHPC_SUCCESS;
    if (!normalized_) return false;
    const uint nch = context_.waveNum;
    if (nch == 1)
        return ophpc_save_bmp(full.c_str(), normalized_[0], w, h, 8, img_.flip, img_.rotate) == OPHPC_SUCCESS;
    if (nch != 3) return false;
    if (img_.merge) {
        // mergeColor (Openholo/src/Openholo.cpp:103-117): channel i -> byte 2-i
        std::vector<uint8_t> rgb((size_t)w * h * 3);
        for (uint c = 0; c < 3; ++c)
            for (size_t i = 0; i < (size_t)w * h; ++i) rgb[i * 3 + (2 - c)] = normalized_[c][i];
        return ophpc_save_bmp(full.c_str(), rgb.data(), w, h, 24, img_.flip, img_.rotate) == OPHPC_SUCCESS;
    }
    bool ok = true;
    for (uint c = 0; c < 3; ++c) {
        const std::string path = dir + std::to_string(c) + "_" + name;
        ok = ophpc_save_bmp(path.c_str(), normalized_[c], w, h, 8, img_.flip, img_.rotate) == OPHPC_SUCCESS && ok;
    }
    return ok;
}

bool ophPointCloud::saveAsOhc(const char* fname) {
    if (fname == nullptr || !complex_H_) return false;
    const uint nch = context_.waveNum;
    const size_t plane = (size_t)buffer_pixels_;
    std::vector<double> field(2 * plane * nch);
    for (uint c = 0; c < nch; ++c)
        std::memcpy(field.data() + 2 * plane * c, complex_H_[c], sizeof(double) * 2 * plane);
    const ophpc_status st = ophpc_save_ohc(fname, field.data(), context_.pixel_number[_X], context_.pixel_number[_Y],
                                           context_.pixel_pitch[_X], context_.pixel_pitch[_Y], nch, wave_length_);
    if (st != OPHPC_SUCCESS) {
        last_error_ = std::string("saveAsOhc: ") + ophpc_status_string(st);
        return false;
    }
    return true;
}

bool ophPointCloud::loadAsOhc(const char* fname) {
    if (fname == nullptr) return false;
    int32_t pnx = 0, pny = 0;
    double ppx = 0, ppy = 0, wl[OPHPC_MAX_CHANNELS] = {0, 0, 0};
    uint32_t nch = 0;
    ophpc_status st = ophpc_load_ohc(fname, &pnx, &pny, &ppx, &ppy, &nch, wl, nullptr, 0);
    if (st != OPHPC_SUCCESS) {
        OPH_LOG("<FAILED> Load ohc : %s\n", fname);
        last_error_ = std::string("loadAsOhc: ") + ophpc_status_string(st);
        return false;
    }
    const size_t plane = (size_t)pnx * (size_t)pny;
    std::vector<double> field(2 * plane * nch);
    st = ophpc_load_ohc(fname, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, field.data(), field.size());
    if (st != OPHPC_SUCCESS) {
        OPH_LOG("<FAILED> Load ohc : %s\n", fname);
        last_error_ = std::string("loadAsOhc: ") + ophpc_status_string(st);
        return false;
    }
    context_.waveNum = nch;
    for (uint i = 0; i < OPHPC_MAX_CHANNELS; ++i) wave_length_[i] = i < nch ? wl[i] : 0.0;
    context_.pixel_number[_X] = pnx;
    context_.pixel_number[_Y] = pny;
    context_.pixel_pitch[_X] = ppx;
    context_.pixel_pitch[_Y] = ppy;
    context_.ss[_X] = pnx * ppx;
    context_.ss[_Y] = pny * ppy;
    context_.k = (2 * kPi) / wave_length_[0];
    if (!initialize()) {
        last_error_ = "loadAsOhc: invalid pixel number or channel count";
        return false;
    }
    for (uint c = 0; c < nch; ++c)
        std::memcpy(complex_H_[c], field.data() + 2 * plane * c, sizeof(double) * 2 * plane);
    encoded_valid_ = false;
    return true;
}

// ------------------------------------------------------------------ C ABI

struct ophpc_pc {
    ophPointCloud* obj;
};

extern "C" {

ophpc_pc* ophpc_pc_create(void) {
    auto* h = new (std::nothrow) ophpc_pc;
    if (!h) return nullptr;
    h->obj = new (std::nothrow) ophPointCloud();
    if (!h->obj) {
        delete h;
        return nullptr;
    }
    return h;
}

void ophpc_pc_release(ophpc_pc* h) {
    if (!h) return;
    h->obj->release();
    delete h;
}

int32_t ophpc_pc_read_config(ophpc_pc* h, const char* path) { return h && h->obj->readConfig(path) ? 1 : 0; }

int64_t ophpc_pc_load_point_cloud(ophpc_pc* h, const char* path) { return h ? h->obj->loadPointCloud(path) : -1; }

void ophpc_pc_set_point_cloud(ophpc_pc* h, const ophpc_vertex* v, uint64_t n) {
    if (!h) return;
    h->obj->setNumberOfPoints(n);
    h->obj->setPointCloudModel(reinterpret_cast<Vertex*>(const_cast<ophpc_vertex*>(v)));
}

void ophpc_pc_set_mode(ophpc_pc* h, uint32_t mode) { if (h) h->obj->SetMode(mode); }
void ophpc_pc_set_viewing_window(ophpc_pc* h, int32_t on) { if (h) h->obj->setViewingWindow(on != 0); }
void ophpc_pc_set_scale(ophpc_pc* h, double sx, double sy, double sz) { if (h) h->obj->setScale(sx, sy, sz); }
void ophpc_pc_set_distance(ophpc_pc* h, double d) { if (h) h->obj->setDistance(d); }
void ophpc_pc_set_offset(ophpc_pc* h, int32_t ox, int32_t oy) { if (h) h->obj->setOffset(ox, oy); }

double ophpc_pc_generate_hologram(ophpc_pc* h, uint32_t diff_flag) {
    return h ? h->obj->generateHologram(diff_flag) : 0.0;
}

void ophpc_pc_encoding(ophpc_pc* h, uint32_t flag) { if (h) h->obj->encoding(flag); }
void ophpc_pc_encoding_passband(ophpc_pc* h, uint32_t flag, uint32_t passband) {
    if (h) h->obj->encoding(flag, passband);
}
void ophpc_pc_normalize(ophpc_pc* h) { if (h) h->obj->normalize(); }

int32_t ophpc_pc_save(ophpc_pc* h, const char* path, uint8_t bits_per_pixel) {
    return h && h->obj->save(path, bits_per_pixel) ? 1 : 0;
}

int32_t ophpc_pc_save_ohc(ophpc_pc* h, const char* path) { return h && h->obj->saveAsOhc(path) ? 1 : 0; }
int32_t ophpc_pc_load_ohc(ophpc_pc* h, const char* path) { return h && h->obj->loadAsOhc(path) ? 1 : 0; }

int32_t ophpc_pc_get_config(ophpc_pc* h, ophpc_config* out) {
    if (!h || !out) return 0;
    h->obj->fillConfig(out);
    return 1;
}

uint64_t ophpc_pc_number_of_points(ophpc_pc* h) { return h ? h->obj->getNumberOfPoints() : 0; }

const ophpc_vertex* ophpc_pc_point_cloud(ophpc_pc* h) {
    return h ? reinterpret_cast<const ophpc_vertex*>(h->obj->getPointCloudModel()) : nullptr;
}

const double* ophpc_pc_complex_field(ophpc_pc* h, uint32_t ch) {
    if (!h || !h->obj->getComplexField() || ch >= h->obj->getContext().waveNum) return nullptr;
    return reinterpret_cast<const double*>(h->obj->getComplexField()[ch]);
}

const double* ophpc_pc_encoded(ophpc_pc* h, uint32_t ch) {
    if (!h || !h->obj->getEncodedBuffer() || ch >= h->obj->getContext().waveNum) return nullptr;
    return h->obj->getEncodedBuffer()[ch];
}

const uint8_t* ophpc_pc_normalized(ophpc_pc* h, uint32_t ch) {
    if (!h || !h->obj->getNormalizedBuffer() || ch >= h->obj->getContext().waveNum) return nullptr;
    return h->obj->getNormalizedBuffer()[ch];
}

const char* ophpc_pc_last_error(ophpc_pc* h) { return h ? h->obj->lastError() : ""; }

}  // extern "C"
