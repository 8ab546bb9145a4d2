/*
 * ophPointCloud — C++ drop-in for Openholo's point-cloud hologram class
 * (ophgen/src/ophPointCloud.h:547-698 with the ophGen / Openholo members it
 * uses), backed by the GB300 kernels of libophpc.
 *
 * Same call sequence as the reference (Example/examPointCloud/
 * examPointCloud.cpp:54-132):
 *
 *   ophPointCloud* h = new ophPointCloud();
 *   h->readConfig("PointCloud.xml");
 *   h->loadPointCloud("cloud.ply");            // or setNumberOfPoints + setPointCloudModel
 *   h->SetMode(MODE_GPU);
 *   h->generateHologram(ophPointCloud::PC_DIFF_RS);
 *   h->encoding(ophPointCloud::ENCODE_PHASE);
 *   h->normalize();
 *   h->save("hologram.bmp");
 *   h->release();
 *
 * Differences from the reference, all deliberate:
 *   - every generateHologram runs on the GPU (MODE_CPU selects nothing: there
 *     is no CPU path); MODE_FLOAT / MODE_FASTMATH select nothing either — one
 *     kernel per method, FP32 arithmetic with FP64 phase reduction, FP64
 *     output; OPHPC_MODE_TENSOR_* selects the tensor-core Fresnel kernel
 *     and, with PC_DIFF_RS, OPHPC_MODE_TENSOR_BF16X3 the tensor-core RS;
 *   - errors are reported through return values and lastError(), never by
 *     exiting the process;
 *   - encoding() supports ENCODE_PHASE, ENCODE_AMPLITUDE, ENCODE_REAL,
 *     ENCODE_IMAGINARY, ENCODE_SIMPLENI, ENCODE_BURCKHARDT and
 *     ENCODE_TWOPHASE on the GPU, and encoding(flag, passband) ENCODE_SSB
 *     and ENCODE_OFFSSB (FP64 FFTs on the GPU, computing what the
 *     reference's code describes: its own FFTW buffers alias the arrays it
 *     shifts); the binary encoders log and do nothing, as an unknown flag
 *     does in the reference.
 */
#ifndef OPHPC_OPHPOINTCLOUD_H
#define OPHPC_OPHPOINTCLOUD_H

#include "ophpc.h"
#include "ophpc_io.h"

#include <complex>
#include <cstdint>
#include <string>

#ifndef MODE_CPU
#define MODE_CPU OPHPC_MODE_CPU
#define MODE_GPU OPHPC_MODE_GPU
#define MODE_DOUBLE OPHPC_MODE_DOUBLE
#define MODE_FLOAT OPHPC_MODE_FLOAT
#define MODE_FASTMATH OPHPC_MODE_FASTMATH
#endif

#ifndef _X
#define _X 0
#define _Y 1
#define _Z 2
#endif

typedef double Real;
typedef unsigned char uchar;
typedef unsigned int uint;
typedef unsigned long long ulonglong;

namespace oph {
/* Complex<T> of Openholo/src/complex.h:82-123: std::complex plus the
 * accessors the path uses. */
template <typename T = double>
class Complex : public std::complex<T> {
public:
    using std::complex<T>::complex;
    Complex() : std::complex<T>() {}
    Complex(const std::complex<T>& c) : std::complex<T>(c) {}
    T mag2() const { return this->real() * this->real() + this->imag() * this->imag(); }
    T mag() const { return std::sqrt(mag2()); }
    T angle() const { return std::atan2(this->imag(), this->real()); }
};
/* vec2 of Openholo/src/ivec.h, as far as the SSB encoder's arguments use
 * it: two Reals indexable with _X, _Y. */
struct vec2 {
    Real v[2];
    vec2(Real a = 0, Real b = 0) : v{a, b} {}
    Real& operator[](int i) { return v[i]; }
    const Real& operator[](int i) const { return v[i]; }
};
}  // namespace oph
using oph::Complex;
using oph::vec2;

/* Vertex (Openholo/src/struct.h:86-106), layout-identical to ophpc_vertex. */
#pragma pack(push, 1)
struct Point { Real pos[3]; };
struct Color { Real color[3]; };
struct Vertex { Point point; Color color; Real phase; };
#pragma pack(pop)
static_assert(sizeof(Vertex) == sizeof(ophpc_vertex), "Vertex must stay 56 bytes");

/* OphConfig (Openholo/src/Openholo.h:96-120), with plain arrays for the
 * ivec2 / vec2 / vec3 members (indexable with _X, _Y, _Z as before). */
struct OphConfig {
    bool bUseDP = true;
    int pixel_number[2] = {0, 0};
    int offset[2] = {0, 0};
    Real pixel_pitch[2] = {0, 0};
    Real shift[3] = {0, 0, 0};
    Real k = 0;
    Real ss[2] = {0, 0};
    uint waveNum = 0;
    Real* wave_length = nullptr;
};

class ophPointCloud {
public:
    enum PC_DIFF_FLAG : int8_t { PC_DIFF_RS = 0x00, PC_DIFF_FRESNEL = 0x01 };
    enum SSB_PASSBAND { SSB_LEFT, SSB_RIGHT, SSB_TOP, SSB_BOTTOM };
    enum ENCODE_FLAG {
        ENCODE_PHASE, ENCODE_AMPLITUDE, ENCODE_REAL, ENCODE_IMAGINARY, ENCODE_SIMPLENI, ENCODE_BURCKHARDT,
        ENCODE_TWOPHASE, ENCODE_SSB, ENCODE_OFFSSB, ENCODE_SIMPLEBINARY, ENCODE_EDBINARY
    };

    explicit ophPointCloud(void);
    explicit ophPointCloud(const char* pc_file, const char* cfg_file);

    /* Base::release (Openholo/src/Base.h:88-96): frees the object. */
    void release(void);

    bool readConfig(const char* cfg_file);
    int loadPointCloud(const char* pc_file);

    void setScale(Real sx, Real sy, Real sz) { scale_[0] = sx; scale_[1] = sy; scale_[2] = sz; }
    void setDistance(Real distance) { distance_ = distance; }
    void setPointCloudModel(Vertex* vertex);
    void setNumberOfPoints(ulonglong n_points) { n_points_ = n_points; }
    void getScale(Real scale[3]) const { scale[0] = scale_[0]; scale[1] = scale_[1]; scale[2] = scale_[2]; }
    Real getDistance(void) const { return distance_; }
    Vertex* getPointCloudModel() { return vertices_; }
    ulonglong getNumberOfPoints() const { return n_points_; }

    void SetMode(unsigned int mode) { mode_ = mode; }
    unsigned int getMode() const { return mode_; }
    bool isCPU() const { return (mode_ & MODE_GPU) ? false : true; }
    void setViewingWindow(bool is_ViewingWindow) { viewing_window_ = is_ViewingWindow; }

    /* Openholo setters used by programs that build the config in code. */
    void setPixelNumber(int nx, int ny);
    void setPixelPitch(Real px, Real py);
    void setWaveLength(Real w, uint idx = 0);
    void setWaveNum(uint n);
    void setOffset(int ox, int oy) { context_.offset[_X] = ox; context_.offset[_Y] = oy; }
    void setFieldLength(Real f) { field_length_ = f; }

    /* Returns the elapsed seconds, 0.0 on a bad flag or a failure. */
    Real generateHologram(uint diff_flag = PC_DIFF_RS);
    void encoding(unsigned int ENCODE_FLAG);
    /* ophPointCloud::encoding(flag, passband) (ophPointCloud.cpp:247-251):
     * ENCODE_SSB runs encodeHologram(), ENCODE_OFFSSB the off-axis
     * single-sideband encoding of channel 0's field into every channel;
     * other flags do nothing. */
    void encoding(unsigned int ENCODE_FLAG, unsigned int SSB_PASSBAND);
    /* ophPointCloud::encodeHologram (ophPointCloud.cpp:191-240); band_limit
     * is not used, as in the reference. */
    void encodeHologram(const vec2 band_limit = vec2(0.8, 0.5), const vec2 spectrum_shift = vec2(0.0, 0.5));
    void normalize(void);
    bool save(const char* fname, uint8_t bitsperpixel = 8, uchar* src = nullptr, uint px = 0, uint py = 0);
    /* Openholo::saveAsOhc / loadAsOhc (Openholo/src/Openholo.cpp:252-319):
     * the complex field with its pitch and wavelengths. loadAsOhc replaces
     * the pixel number, pitch and wavelengths of the context and the
     * complex field; the encoded and normalized buffers restart at zero. */
    bool saveAsOhc(const char* fname);
    bool loadAsOhc(const char* fname);

    Complex<Real>** getComplexField(void) { return complex_H_; }
    Real** getEncodedBuffer(void) { return encoded_; }
    uchar** getNormalizedBuffer(void) { return normalized_; }
    OphConfig& getContext(void) { return context_; }
    uint* getProgress() { return &progress_; }

    /* GB300 additions (no reference counterpart). */
    const char* lastError() const { return last_error_.c_str(); }
    ophpc_context* gpuContext() const { return gpu_; }
    void fillConfig(ophpc_config* out) const;

protected:
    virtual ~ophPointCloud(void);

private:
    bool initialize();          /* ophGen::initialize: host buffers per channel */
    void freeBuffers();
    bool ensureGpu();
    bool ensureDevice(size_t bytes_vertices, size_t bytes_field, size_t bytes_encoded, size_t bytes_codes);
    bool ensureStreams();
    void encodeSideband(unsigned int flag, unsigned int passband, Real shift_x, Real shift_y);

    OphConfig context_;
    Real wave_length_[OPHPC_MAX_CHANNELS] = {0, 0, 0};
    ophpc_image_config img_{};
    Real scale_[3] = {1, 1, 1};
    Real distance_ = 0;
    Real field_length_ = 0;
    bool viewing_window_ = false;
    unsigned int mode_ = 0;
    uint progress_ = 0;
    uint n_old_channels_ = 0;
    long long buffer_pixels_ = 0;
    ulonglong n_points_ = 0;
    Vertex* vertices_ = nullptr;
    ulonglong vertices_cap_ = 0;   /* records vertices_ holds */
    bool vertices_pinned_ = false; /* vertices_ is page-locked (cudaHostAlloc) */
    Complex<Real>** complex_H_ = nullptr;
    Real** encoded_ = nullptr;
    uchar** normalized_ = nullptr;
    std::string last_error_;

    ophpc_context* gpu_ = nullptr;
    void* d_vertices_ = nullptr;
    void* d_field_ = nullptr;
    void* d_encoded_ = nullptr;
    void* d_codes_ = nullptr;
    size_t cap_v_ = 0, cap_f_ = 0, cap_e_ = 0, cap_c_ = 0;
    bool encoded_valid_ = false;
    bool host_pinned_ = false;  /* per-channel buffers are page-locked (cudaHostAlloc) */
    void* streams_[OPHPC_MAX_CHANNELS] = {};   /* encoding(): one CUDA stream per channel */
};

#endif /* OPHPC_OPHPOINTCLOUD_H */
