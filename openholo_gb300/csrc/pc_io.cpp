// Host-side files of the point-cloud path: flat-XML config, PLY point clouds
// and BMP holograms (declared in include/ophpc_io.h).
//
// Behaviour follows the reference where it is defined:
//   config  ophgen/src/ophGen.cpp:221-358, ophgen/src/ophPointCloud.cpp:83-149
//           (tinyxml2 Query*Text semantics; the first node of the document
//           must be the root element, as xml_doc.FirstChild() requires)
//   PLY     Openholo/src/PLYparser.cpp:142-449 (ASCII coordinates as double,
//           binary float coordinates, phase rounded through float, colours
//           (double)(c / 255.f), 0.5 everywhere without a `color channel`
//           element)
//   BMP     Openholo/src/Openholo.cpp:135-251 (8-bit grey palette, rows in
//           buffer order, 4-byte row padding)
// and is made well defined where the reference's is not: big-endian binary
// PLY is byte-swapped, double-typed binary properties are read as doubles,
// flips and the 180-degree rotation work on a separate buffer.
#include "ophpc_io.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------------ XML

bool ends_with(const std::string& s, const std::string& e) {
    // Openholo::checkExtension: the text from the last '.' must equal ext
    const size_t dot = s.find_last_of('.');
    if (dot == std::string::npos) return false;
    return s.compare(dot, std::string::npos, e) == 0;
}

// Children of the root element: name -> text of the first element with
// that name. Returns false when the document does not start with an
// element (declaration, comment or text first) or is malformed.
bool parse_flat_xml(const std::string& doc, std::map<std::string, std::string>& kv) {
    size_t i = 0;
    auto skip_ws = [&]() {
        while (i < doc.size() && std::isspace((unsigned char)doc[i])) ++i;
    };
    skip_ws();
    if (i >= doc.size() || doc[i] != '<') return false;
    if (doc.compare(i, 2, "<?") == 0 || doc.compare(i, 4, "<!--") == 0 || doc.compare(i, 2, "<!") == 0)
        return false;
    // root start tag
    size_t gt = doc.find('>', i);
    if (gt == std::string::npos) return false;
    std::string root_tag = doc.substr(i + 1, gt - i - 1);
    if (!root_tag.empty() && root_tag.back() == '/') return true;   // empty root
    std::string root_name = root_tag.substr(0, root_tag.find_first_of(" \t\r\n"));
    i = gt + 1;
    const std::string root_close = "</" + root_name;
    while (i < doc.size()) {
        size_t lt = doc.find('<', i);
        if (lt == std::string::npos) return false;
        i = lt;
        if (doc.compare(i, 4, "<!--") == 0) {
            size_t e = doc.find("-->", i + 4);
            if (e == std::string::npos) return false;
            i = e + 3;
            continue;
        }
        if (doc.compare(i, root_close.size(), root_close) == 0) return true;
        if (doc.compare(i, 2, "</") == 0) return false;   // stray close tag
        gt = doc.find('>', i);
        if (gt == std::string::npos) return false;
        std::string tag = doc.substr(i + 1, gt - i - 1);
        const bool self_close = !tag.empty() && tag.back() == '/';
        std::string name = tag.substr(0, tag.find_first_of(" \t\r\n/"));
        i = gt + 1;
        if (self_close) {
            kv.emplace(name, std::string());   // no text: queries fail
            continue;
        }
        // text up to the next tag; skip any nested content to the close tag
        size_t next = doc.find('<', i);
        if (next == std::string::npos) return false;
        std::string text = doc.substr(i, next - i);
        const std::string close = "</" + name + ">";
        size_t end = doc.find(close, i);
        if (end == std::string::npos) return false;
        kv.emplace(name, text);   // first element of a name wins
        i = end + close.size();
    }
    return false;
}

// tinyxml2 XMLUtil::ToInt / ToDouble / ToBool equivalents: a numeric prefix
// after optional whitespace ("%d", "%lf", hex "0x.." for ints).
bool to_int(const std::string& s, int* v) {
    const char* p = s.c_str();
    while (*p && std::isspace((unsigned char)*p)) ++p;
    char* end = nullptr;
    errno = 0;
    long r;
    if (p[0] == '0' && (p[1] == 'x' || p[1] == 'X'))
        r = std::strtol(p + 2, &end, 16);
    else
        r = std::strtol(p, &end, 10);
    if (end == p || errno == ERANGE || r > INT32_MAX || r < INT32_MIN) return false;
    *v = (int)r;
    return true;
}

bool to_double(const std::string& s, double* v) {
    const char* p = s.c_str();
    while (*p && std::isspace((unsigned char)*p)) ++p;
    char* end = nullptr;
    double r = std::strtod(p, &end);
    if (end == p) return false;
    *v = r;
    return true;
}

bool to_bool(const std::string& s, bool* v) {
    int iv;
    if (to_int(s, &iv)) {
        *v = iv != 0;
        return true;
    }
    std::string t = s;
    t.erase(0, t.find_first_not_of(" \t\r\n"));
    t.erase(t.find_last_not_of(" \t\r\n") + 1);
    if (t == "true" || t == "True" || t == "TRUE") {
        *v = true;
        return true;
    }
    if (t == "false" || t == "False" || t == "FALSE") {
        *v = false;
        return true;
    }
    return false;
}

// ------------------------------------------------------------------ PLY

enum class PT { I8, U8, I16, U16, I32, U32, F32, F64, INVALID };

PT ptype(const std::string& t) {
    if (t == "int8" || t == "char") return PT::I8;
    if (t == "uint8" || t == "uchar") return PT::U8;
    if (t == "int16" || t == "short") return PT::I16;
    if (t == "uint16" || t == "ushort") return PT::U16;
    if (t == "int32" || t == "int") return PT::I32;
    if (t == "uint32" || t == "uint") return PT::U32;
    if (t == "float32" || t == "float") return PT::F32;
    if (t == "float64" || t == "double" || t == "real") return PT::F64;
    return PT::INVALID;
}

int psize(PT t) {
    switch (t) {
        case PT::I8: case PT::U8: return 1;
        case PT::I16: case PT::U16: return 2;
        case PT::I32: case PT::U32: case PT::F32: return 4;
        case PT::F64: return 8;
        default: return 0;
    }
}

struct Prop {
    std::string name;
    PT type = PT::INVALID;
    bool is_list = false;
    PT list_type = PT::INVALID;
};

struct Elem {
    std::string name;
    uint64_t size = 0;
    std::vector<Prop> props;
    int find(const std::string& n) const {
        for (size_t j = 0; j < props.size(); ++j)
            if (props[j].name == n) return (int)j;
        return -1;
    }
};

bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

inline double colour(int c) { return (double)((float)c / 255.f); }

// Decodes one binary scalar of type t at p (byte-swapped if needed).
inline double decode_scalar(const unsigned char* p, PT t, bool swap) {
    unsigned char b[8];
    const int n = psize(t);
    std::memcpy(b, p, (size_t)n);
    if (swap) std::reverse(b, b + n);
    switch (t) {
        case PT::I8: { int8_t v; std::memcpy(&v, b, 1); return v; }
        case PT::U8: return b[0];
        case PT::I16: { int16_t v; std::memcpy(&v, b, 2); return v; }
        case PT::U16: { uint16_t v; std::memcpy(&v, b, 2); return v; }
        case PT::I32: { int32_t v; std::memcpy(&v, b, 4); return v; }
        case PT::U32: { uint32_t v; std::memcpy(&v, b, 4); return v; }
        case PT::F32: { float v; std::memcpy(&v, b, 4); return v; }
        case PT::F64: { double v; std::memcpy(&v, b, 8); return v; }
        default: return 0.0;
    }
}

struct PlyHeader {
    bool binary = false, big = false;
    std::vector<Elem> elems;
    int iv = -1, ic = -1, ifc = -1;
};

// Header up to and including `end_header`; f is left at the first data byte.
bool parse_ply_header(std::ifstream& f, PlyHeader& h) {
    std::string line, tok;
    if (!std::getline(f, line)) return false;
    {
        std::istringstream ls(line);
        ls >> tok;
        if (tok != "ply" && tok != "PLY") return false;
    }
    bool header_done = false;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        tok.clear();
        ls >> tok;
        if (tok == "format") {
            std::string fmt;
            ls >> fmt;
            if (fmt == "binary_little_endian") h.binary = true;
            else if (fmt == "binary_big_endian") h.binary = h.big = true;
        } else if (tok == "element") {
            Elem e;
            ls >> e.name >> e.size;
            h.elems.push_back(e);
        } else if (tok == "property") {
            if (h.elems.empty()) return false;
            Prop p;
            std::string t;
            ls >> t;
            if (t == "list") {
                std::string ct;
                ls >> ct >> t;
                p.is_list = true;
                p.list_type = ptype(ct);
            }
            p.type = ptype(t);
            ls >> p.name;
            h.elems.back().props.push_back(p);
        } else if (tok == "end_header") {
            header_done = true;
            break;
        }
    }
    if (!header_done) return false;
    for (size_t k = 0; k < h.elems.size(); ++k) {
        if (h.iv < 0 && h.elems[k].name == "vertex") h.iv = (int)k;
        if (h.ic < 0 && h.elems[k].name == "color") h.ic = (int)k;
        if (h.ifc < 0 && h.elems[k].name == "face") h.ifc = (int)k;
    }
    if (h.iv < 0) return false;
    const Elem& V = h.elems[h.iv];
    if (V.find("x") < 0 || V.find("y") < 0 || V.find("z") < 0) return false;
    if (V.size > (uint64_t)INT32_MAX) return false;
    return true;
}

// Whole-file PLY reader. The header is parsed line by line; the data are
// read in one block and decoded in place: an element without list
// properties has a fixed record size, so its records are decoded at
// precomputed offsets; elements with lists (faces) are walked record by
// record. ASCII records are one line each, tokens split on whitespace.
// out must hold the header's vertex count.
int64_t load_ply(const char* path_in, ophpc_vertex* out, bool count_only) {
    if (!path_in) return -1;
    std::string path = path_in;
    if (path.find(".ply") == std::string::npos && path.find(".PLY") == std::string::npos) path += ".ply";
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f.is_open()) return -1;
    PlyHeader h;
    if (!parse_ply_header(f, h)) return -1;
    const Elem& V = h.elems[h.iv];
    const uint64_t n = V.size;
    if (count_only) return (int64_t)n;

    const int px = V.find("x"), py = V.find("y"), pz = V.find("z");
    const bool found_channel = h.ic >= 0 && h.elems[h.ic].find("channel") >= 0;
    const bool found_face = h.ifc >= 0 && h.elems[h.ifc].find("vertex_indices") >= 0;
    int pr = V.find("red"), pg = V.find("green"), pb = V.find("blue");
    if (pb < 0) {
        pr = V.find("diffuse_red");
        pg = V.find("diffuse_green");
        pb = V.find("diffuse_blue");
    }
    const int pphase = V.find("phase");
    int fr = -1, fg = -1, fb = -1;
    if (h.ifc >= 0) {
        fr = h.elems[h.ifc].find("red");
        fg = h.elems[h.ifc].find("green");
        fb = h.elems[h.ifc].find("blue");
    }
    std::memset(out, 0, sizeof(ophpc_vertex) * (size_t)n);

    // the data block
    const std::streampos data_at = f.tellg();
    f.seekg(0, std::ios::end);
    const std::streampos file_end = f.tellg();
    f.seekg(data_at);
    const size_t nbytes = (size_t)(file_end - data_at);
    std::string data(nbytes + 1, '\0');
    if (nbytes && !f.read(&data[0], (std::streamsize)nbytes)) return -1;
    const unsigned char* q = (const unsigned char*)data.data();
    const unsigned char* const qend = q + nbytes;
    const bool swap = h.binary && (h.big == host_little_endian());

    auto put_vertex = [&](uint64_t e, const double* vals, bool binary) {
        ophpc_vertex& vx = out[e];
        if (binary) {   // binary coordinates land in a float in the reference
            vx.pos[0] = V.props[px].type == PT::F64 ? vals[px] : (double)(float)vals[px];
            vx.pos[1] = V.props[py].type == PT::F64 ? vals[py] : (double)(float)vals[py];
            vx.pos[2] = V.props[pz].type == PT::F64 ? vals[pz] : (double)(float)vals[pz];
        } else {
            vx.pos[0] = vals[px];
            vx.pos[1] = vals[py];
            vx.pos[2] = vals[pz];
        }
        if (!found_face) {
            vx.color[0] = colour(pr >= 0 ? (int)vals[pr] : 0);
            vx.color[1] = colour(pg >= 0 ? (int)vals[pg] : 0);
            vx.color[2] = colour(pb >= 0 ? (int)vals[pb] : 0);
        }
        if (pphase >= 0) vx.phase = (double)(float)vals[pphase];
    };
    auto put_face = [&](uint64_t e, const double* vals) {
        if (e >= n || fb < 0) return;
        ophpc_vertex& vx = out[e];
        vx.color[0] = colour(fr >= 0 ? (int)vals[fr] : 0);
        vx.color[1] = colour(fg >= 0 ? (int)vals[fg] : 0);
        vx.color[2] = colour((int)vals[fb]);
    };

    std::vector<double> vals;
    for (size_t k = 0; k < h.elems.size(); ++k) {
        const Elem& E = h.elems[k];
        const size_t np = E.props.size();
        vals.assign(np, 0.0);
        if (h.binary) {
            bool fixed = true;
            size_t stride = 0;
            std::vector<size_t> off(np);
            for (size_t j = 0; j < np; ++j) {
                if (E.props[j].is_list || psize(E.props[j].type) == 0) fixed = false;
                off[j] = stride;
                stride += (size_t)psize(E.props[j].type);
            }
            if (fixed) {
                if (E.size > (uint64_t)(qend - q) / (stride ? stride : 1)) return -1;
                if ((int)k == h.iv) {
                    // only the properties a vertex record uses, decoded in
                    // parallel over record ranges
                    const int want[7] = {px, py, pz, pr, pg, pb, pphase};
                    const unsigned char* base = q;
                    auto decode_range = [&](uint64_t e0, uint64_t e1) {
                        double vv[64];
                        std::vector<double> big(np > 64 ? np : 0);
                        double* vr = np > 64 ? big.data() : vv;
                        for (size_t j = 0; j < np; ++j) vr[j] = 0.0;
                        for (uint64_t e = e0; e < e1; ++e) {
                            const unsigned char* r = base + e * stride;
                            for (int w : want)
                                if (w >= 0) vr[w] = decode_scalar(r + off[w], E.props[w].type, swap);
                            put_vertex(e, vr, true);
                        }
                    };
                    const uint64_t per = 1u << 16;
                    const unsigned nt = (unsigned)std::min<uint64_t>(
                        std::max(1u, std::min(16u, std::thread::hardware_concurrency())), (E.size + per - 1) / per);
                    if (nt <= 1) {
                        decode_range(0, E.size);
                    } else {
                        std::vector<std::thread> th;
                        const uint64_t chunk = (E.size + nt - 1) / nt;
                        for (unsigned t = 0; t < nt; ++t) {
                            const uint64_t e0 = t * chunk, e1 = std::min<uint64_t>(E.size, e0 + chunk);
                            if (e0 < e1) th.emplace_back(decode_range, e0, e1);
                        }
                        for (auto& t : th) t.join();
                    }
                } else if ((int)k == h.ifc) {
                    for (uint64_t e = 0; e < E.size; ++e) {
                        const unsigned char* r = q + e * stride;
                        for (size_t j = 0; j < np; ++j) vals[j] = decode_scalar(r + off[j], E.props[j].type, swap);
                        put_face(e, vals.data());
                    }
                }
                q += stride * E.size;
                continue;
            }
            for (uint64_t e = 0; e < E.size; ++e) {
                std::fill(vals.begin(), vals.end(), 0.0);
                for (size_t j = 0; j < np; ++j) {
                    const Prop& p = E.props[j];
                    if (p.is_list) {
                        const int cs = psize(p.list_type), es = psize(p.type);
                        if (cs == 0 || es == 0 || qend - q < cs) return -1;
                        const double cnt = decode_scalar(q, p.list_type, swap);
                        q += cs;
                        if (!(cnt >= 0) || cnt * es > (double)(qend - q)) return -1;
                        q += (size_t)cnt * (size_t)es;
                        continue;
                    }
                    const int sz = psize(p.type);
                    if (sz == 0 || qend - q < sz) return -1;
                    vals[j] = decode_scalar(q, p.type, swap);
                    q += sz;
                }
                if ((int)k == h.iv) put_vertex(e, vals.data(), true);
                else if ((int)k == h.ifc) put_face(e, vals.data());
            }
        } else {
            for (uint64_t e = 0; e < E.size; ++e) {
                if (q >= qend) return -1;   // a missing line
                const unsigned char* eol = (const unsigned char*)std::memchr(q, '\n', (size_t)(qend - q));
                if (!eol) eol = qend;
                std::fill(vals.begin(), vals.end(), 0.0);
                const char* c = (const char*)q;
                const char* le = (const char*)eol;
                for (size_t j = 0; j < np; ++j) {
                    while (c < le && std::isspace((unsigned char)*c)) ++c;
                    if (c >= le) break;
                    const char* t0 = c;
                    while (c < le && !std::isspace((unsigned char)*c)) ++c;
                    const std::string tok(t0, c);
                    const Prop& p = E.props[j];
                    if (p.type == PT::F32 || p.type == PT::F64) vals[j] = std::strtod(tok.c_str(), nullptr);
                    else vals[j] = (double)std::strtol(tok.c_str(), nullptr, 10);
                    if (p.is_list) break;   // lists in ASCII carry no vertex data we read
                }
                if ((int)k == h.iv) put_vertex(e, vals.data(), false);
                else if ((int)k == h.ifc) put_face(e, vals.data());
                q = eol < qend ? eol + 1 : qend;
            }
        }
    }
    if (!found_channel)
        for (uint64_t e = 0; e < n; ++e) out[e].color[0] = out[e].color[1] = out[e].color[2] = 0.5;
    return (int64_t)n;
}

// ------------------------------------------------------------------ BMP

void put16(std::vector<uint8_t>& b, size_t at, uint16_t v) {
    b[at] = (uint8_t)(v & 0xff);
    b[at + 1] = (uint8_t)(v >> 8);
}
void put32(std::vector<uint8_t>& b, size_t at, uint32_t v) {
    for (int i = 0; i < 4; ++i) b[at + i] = (uint8_t)(v >> (8 * i));
}

// ------------------------------------------------------------------ OHC

// Field-info header of the .ohc format (65 bytes, packed, little-endian).
#pragma pack(push, 1)
struct OhcFileHeader {
    char signature[2];
    uint64_t file_size;
    uint8_t version_major, version_minor;
    uint32_t reserved1, reserved2;
    uint32_t off_bytes;
};
struct OhcFieldInfo {
    uint32_t header_size;
    uint32_t px_x, px_y;
    double pitch_x, pitch_y;
    uint8_t pitch_unit;
    uint32_t n_wavelengths;
    uint8_t color_type, color_arrange, wavelength_unit, data_type, store, code_type, phase_coded;
    double phase_min, phase_max;
    uint64_t field_bytes;
    uint8_t compression;
};
#pragma pack(pop)
static_assert(sizeof(OhcFileHeader) == 24, "ohc file header");
static_assert(sizeof(OhcFieldInfo) == 65, "ohc field info header");

std::string ohc_path(const char* p) {
    std::string s = p;
    if (!ends_with(s, ".ohc")) s += ".ohc";
    return s;
}

}  // namespace

extern "C" {

ophpc_status ophpc_save_ohc(const char* path, const double* field, int32_t pnx, int32_t pny, double ppx, double ppy,
                            uint32_t nch, const double* wavelengths) {
    if (!path || !field || !wavelengths || pnx <= 0 || pny <= 0 || nch < 1 || nch > OPHPC_MAX_CHANNELS)
        return OPHPC_ERROR_INVALID_ARGUMENT;
    const uint64_t npx = (uint64_t)pnx * (uint64_t)pny;
    OhcFieldInfo fi;
    std::memset(&fi, 0, sizeof(fi));
    fi.header_size = (uint32_t)(sizeof(OhcFieldInfo) + 8 * nch);
    fi.px_x = (uint32_t)pnx;
    fi.px_y = (uint32_t)pny;
    fi.pitch_x = ppx;
    fi.pitch_y = ppy;
    fi.pitch_unit = 1;           // metre
    fi.n_wavelengths = nch;
    fi.color_type = 2;           // multiple colours
    fi.color_arrange = 2;        // one plane per channel
    fi.wavelength_unit = 1;      // metre
    fi.data_type = 10;           // float64
    fi.store = 1;                // stored directly
    fi.code_type = 2;            // real & imaginary
    fi.phase_coded = 0;
    fi.phase_min = -1.0;
    fi.phase_max = 1.0;
    fi.field_bytes = 16 * npx * nch;
    fi.compression = 0;
    OhcFileHeader fh;
    fh.signature[0] = 'O';
    fh.signature[1] = 'H';
    fh.version_major = 3;
    fh.version_minor = 0;
    fh.reserved1 = fh.reserved2 = 0;
    fh.off_bytes = (uint32_t)(sizeof(OhcFileHeader) + fi.header_size);
    fh.file_size = fh.off_bytes + fi.field_bytes;
    FILE* fp = std::fopen(ohc_path(path).c_str(), "wb");
    if (!fp) return OPHPC_ERROR_IO;
    bool ok = std::fwrite(&fh, sizeof(fh), 1, fp) == 1 && std::fwrite(&fi, sizeof(fi), 1, fp) == 1 &&
              std::fwrite(wavelengths, sizeof(double), nch, fp) == nch;
    std::vector<double> plane((size_t)npx);
    for (int part = 0; part < 2 && ok; ++part)
        for (uint32_t c = 0; c < nch && ok; ++c) {
            const double* src = field + (size_t)c * npx * 2;
            for (uint64_t i = 0; i < npx; ++i) plane[i] = src[2 * i + part];
            ok = std::fwrite(plane.data(), sizeof(double), (size_t)npx, fp) == npx;
        }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? OPHPC_SUCCESS : OPHPC_ERROR_IO;
}

ophpc_status ophpc_load_ohc(const char* path, int32_t* pnx, int32_t* pny, double* ppx, double* ppy, uint32_t* nch_out,
                            double* wavelengths, double* field, uint64_t capacity) {
    if (!path) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::ifstream f(ohc_path(path), std::ios::in | std::ios::binary);
    if (!f.is_open()) return OPHPC_ERROR_IO;
    OhcFileHeader fh;
    OhcFieldInfo fi;
    if (!f.read((char*)&fh, sizeof(fh)) || fh.signature[0] != 'O' || fh.signature[1] != 'H') return OPHPC_ERROR_IO;
    if (!f.read((char*)&fi, sizeof(fi))) return OPHPC_ERROR_IO;
    const uint32_t nch = fi.n_wavelengths;
    if (nch < 1 || nch > OPHPC_MAX_CHANNELS || fi.px_x == 0 || fi.px_y == 0) return OPHPC_ERROR_UNSUPPORTED;
    double wl[OPHPC_MAX_CHANNELS] = {0, 0, 0};
    if (!f.read((char*)wl, sizeof(double) * nch)) return OPHPC_ERROR_IO;
    // pitch and wavelengths as stored, whatever their unit field says
    // (ImgDecoderOhc::getPixelPitch / getWavelength)
    if (pnx) *pnx = (int32_t)fi.px_x;
    if (pny) *pny = (int32_t)fi.px_y;
    if (ppx) *ppx = fi.pitch_x;
    if (ppy) *ppy = fi.pitch_y;
    if (nch_out) *nch_out = nch;
    if (wavelengths)
        for (uint32_t c = 0; c < nch; ++c) wavelengths[c] = wl[c];
    if (!field) return OPHPC_SUCCESS;
    const uint64_t npx = (uint64_t)fi.px_x * fi.px_y;
    if (capacity < 2 * npx * nch) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (fi.store != 1 || (fi.data_type != 9 && fi.data_type != 10)) return OPHPC_ERROR_UNSUPPORTED;
    if (fi.code_type != 1 && fi.code_type != 2) return OPHPC_ERROR_UNSUPPORTED;   // AP or RI
    f.seekg(fh.off_bytes, std::ios::beg);
    const uint64_t nval = 2 * npx * nch;
    std::vector<double> buf((size_t)nval);
    if (fi.data_type == 10) {
        if (!f.read((char*)buf.data(), (std::streamsize)(8 * nval))) return OPHPC_ERROR_IO;
    } else {
        std::vector<float> b32((size_t)nval);
        if (!f.read((char*)b32.data(), (std::streamsize)(4 * nval))) return OPHPC_ERROR_IO;
        for (uint64_t i = 0; i < nval; ++i) buf[i] = b32[i];
    }
    const uint64_t nf = npx * nch;   // values per part
    for (uint32_t c = 0; c < nch; ++c)
        for (uint64_t i = 0; i < npx; ++i) {
            // colour arrangement: 2 = one plane per channel, 1 = channels interleaved per pixel
            const uint64_t k = fi.color_arrange == 1 ? i * nch + c : c * npx + i;
            double a = buf[k], b = buf[nf + k];
            if (fi.code_type == 1) {   // amplitude, phase (the reference leaves the field zero here)
                const double amp = a, ph = b;
                a = amp * std::cos(ph);
                b = amp * std::sin(ph);
            }
            field[2 * (c * npx + i) + 0] = a;
            field[2 * (c * npx + i) + 1] = b;
        }
    return OPHPC_SUCCESS;
}


ophpc_status ophpc_read_config(const char* xml_path, ophpc_config* cfg, ophpc_image_config* img) {
    if (!xml_path || !cfg) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (!ends_with(xml_path, ".xml")) return OPHPC_ERROR_IO;
    std::ifstream f(xml_path, std::ios::in | std::ios::binary);
    if (!f.is_open()) return OPHPC_ERROR_IO;
    std::stringstream ss;
    ss << f.rdbuf();
    std::map<std::string, std::string> kv;
    const bool parsed = parse_flat_xml(ss.str(), kv);
    if (!parsed) return OPHPC_ERROR_IO;

    std::memset(cfg, 0, sizeof(*cfg));
    bool ok = true;
    auto get_i = [&](const char* k, int* v) {
        auto it = kv.find(k);
        return it != kv.end() && to_int(it->second, v);
    };
    auto get_d = [&](const char* k, double* v) {
        auto it = kv.find(k);
        return it != kv.end() && to_double(it->second, v);
    };
    auto get_b = [&](const char* k, bool* v) {
        auto it = kv.find(k);
        return it != kv.end() && to_bool(it->second, v);
    };
    int nwave = 1;
    if (!get_i("SLM_WaveNum", &nwave)) {
        ok = false;
        nwave = 1;
    }
    if (nwave < 1 || nwave > OPHPC_MAX_CHANNELS) {
        ok = false;
        nwave = std::max(1, std::min(nwave, (int)OPHPC_MAX_CHANNELS));
    }
    cfg->n_channels = (uint32_t)nwave;
    for (int w = 1; w <= nwave; ++w) {
        char key[32];
        std::snprintf(key, sizeof(key), "SLM_WaveLength_%d", w);
        if (!get_d(key, &cfg->wave_length[w - 1])) ok = false;
    }
    if (!get_i("SLM_PixelNumX", &cfg->pixel_number[0])) ok = false;
    if (!get_i("SLM_PixelNumY", &cfg->pixel_number[1])) ok = false;
    if (!get_d("SLM_PixelPitchX", &cfg->pixel_pitch[0])) ok = false;
    if (!get_d("SLM_PixelPitchY", &cfg->pixel_pitch[1])) ok = false;
    if (img) {
        bool b;
        img->rotate = get_b("IMG_Rotation", &b) ? b : 0;
        img->merge = get_b("IMG_Merge", &b) ? b : 0;
        int fl;
        img->flip = get_i("IMG_Flip", &fl) ? fl : 0;
        img->double_precision = get_b("DoublePrecision", &b) ? b : 1;
        for (int a = 0; a < 3; ++a) {
            static const char* names[3] = {"ShiftX", "ShiftY", "ShiftZ"};
            double d;
            img->shift[a] = get_d(names[a], &d) ? d : 0.0;
        }
        img->random_phase = get_b("RandomPhase", &b) ? b : 0;
        int ns;
        img->num_of_stream = get_i("NumOfStream", &ns) ? ns : 1;
    }
    {
        double fl;
        cfg->field_length = get_d("FieldLength", &fl) ? fl : 0.0;
    }
    // the reference returns before reading the point-cloud keys when the
    // common part failed (ophPointCloud.cpp:85-86)
    if (!ok) return OPHPC_ERROR_CONFIG;
    if (!get_d("ScaleX", &cfg->scale[0])) ok = false;
    if (!get_d("ScaleY", &cfg->scale[1])) ok = false;
    if (!get_d("ScaleZ", &cfg->scale[2])) ok = false;
    if (!get_d("Distance", &cfg->distance)) ok = false;
    return ok ? OPHPC_SUCCESS : OPHPC_ERROR_CONFIG;
}

int64_t ophpc_load_ply(const char* path, ophpc_vertex* out, uint64_t capacity) {
    if (!out) return load_ply(path, nullptr, true);
    const int64_t n = load_ply(path, nullptr, true);
    if (n < 0) return -1;
    if (capacity >= (uint64_t)n) return load_ply(path, out, false);   // straight into the caller's buffer
    std::vector<ophpc_vertex> v((size_t)n);
    if (load_ply(path, v.data(), false) < 0) return -1;
    std::memcpy(out, v.data(), sizeof(ophpc_vertex) * (size_t)capacity);
    return n;
}

ophpc_status ophpc_save_bmp(const char* path, const uint8_t* pixels, int32_t width, int32_t height,
                            int32_t bpp, int32_t flip, int32_t rotate) {
    if (!path || !pixels || width <= 0 || height <= 0 || (bpp != 8 && bpp != 24))
        return OPHPC_ERROR_INVALID_ARGUMENT;
    const int ch = bpp / 8;
    const size_t row_bytes = (size_t)width * ch;
    const size_t stride = ((row_bytes) + 3) & ~(size_t)3;
    const size_t pix_bytes = stride * (size_t)height;
    const bool palette = bpp <= 8;
    const size_t header = 14 + 40 + (palette ? 256 * 4 : 0);
    const size_t total = header + pix_bytes;
    if (total > 0xffffffffull) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::vector<uint8_t> b(total, 0);
    b[0] = 'B';
    b[1] = 'M';
    put32(b, 2, (uint32_t)total);
    put32(b, 6, 0);
    put32(b, 10, (uint32_t)header);
    put32(b, 14, 40);
    put32(b, 18, (uint32_t)width);
    put32(b, 22, (uint32_t)height);
    put16(b, 26, 1);
    put16(b, 28, (uint16_t)bpp);
    put32(b, 30, 0);
    put32(b, 34, (uint32_t)pix_bytes);
    put32(b, 38, 0);
    put32(b, 42, 0);
    put32(b, 46, palette ? 256 : 0);
    put32(b, 50, 0);
    if (palette)
        for (int i = 0; i < 256; ++i) {
            b[54 + 4 * i + 0] = (uint8_t)i;
            b[54 + 4 * i + 1] = (uint8_t)i;
            b[54 + 4 * i + 2] = (uint8_t)i;
        }
    bool vflip = flip == 1 || flip == 3;
    bool hflip = flip == 2 || flip == 3;
    if (rotate) {   // 180 degrees = both flips
        vflip = !vflip;
        hflip = !hflip;
    }
    for (int y = 0; y < height; ++y) {
        const int sy = vflip ? height - 1 - y : y;
        const uint8_t* src = pixels + (size_t)sy * row_bytes;
        uint8_t* dst = b.data() + header + (size_t)y * stride;
        if (!hflip) {
            std::memcpy(dst, src, row_bytes);
        } else {
            for (int x = 0; x < width; ++x) std::memcpy(dst + (size_t)x * ch, src + (size_t)(width - 1 - x) * ch, ch);
        }
    }
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return OPHPC_ERROR_IO;
    const size_t w = std::fwrite(b.data(), 1, b.size(), fp);
    const int cl = std::fclose(fp);
    return (w == b.size() && cl == 0) ? OPHPC_SUCCESS : OPHPC_ERROR_IO;
}

}  // extern "C"
