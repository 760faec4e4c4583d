// ply_reader.cpp — PLY parsing for the mesh path (host I/O).
//
// Reads what PlyLoader(path) reads (PlyLoader.cpp:66-224) through the
// vendored plyfile library's conversion rules (third-party/plyfile.c):
//   - vertex properties x y z nx ny nz red green blue, each converted to
//     float the way plyfile's get_*_item + store_item do (binary: the stored
//     type read natively, then int -> double -> float or float -> double ->
//     float; ascii: atoi / strtoul / atof, then to float);
//   - face property vertex_indices, the first property of that name, its
//     count and items converted to int;
//   - binary_big_endian files: plyfile reads the bytes in host (little-
//     endian) order and PlyLoader's toHostOrder then swaps every converted
//     float and index (PlyLoader.cpp:104-120, 152, 208-211); the same two
//     steps are applied here, so such files give the reference's values;
//   - other elements and properties are skipped.
// Errors the reference meets with ASSERT/exit or undefined behaviour
// (missing elements, an index outside the vertex array, a truncated file)
// return SVO_ERR_FORMAT or SVO_ERR_IO.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mesh.h"

namespace svo {

namespace {

enum PlyType { kInvalid = 0, kChar, kShort, kInt, kUChar, kUShort, kUInt, kFloat, kDouble };

int type_size(int t) {
    static const int sz[] = {0, 1, 2, 4, 1, 2, 4, 4, 8};
    return sz[t];
}

int parse_type(const std::string &s) {
    if (s == "char" || s == "int8") return kChar;
    if (s == "short" || s == "int16") return kShort;
    if (s == "int" || s == "int32") return kInt;
    if (s == "uchar" || s == "uint8") return kUChar;
    if (s == "ushort" || s == "uint16") return kUShort;
    if (s == "uint" || s == "uint32") return kUInt;
    if (s == "float" || s == "float32") return kFloat;
    if (s == "double" || s == "float64") return kDouble;
    return kInvalid;
}

struct Prop {
    std::string name;
    int type = kInvalid;        // item type
    int count_type = kInvalid;  // != kInvalid for a list
};

struct Elem {
    std::string name;
    uint64_t count = 0;
    std::vector<Prop> props;
};

// plyfile's (int, uint, double) triple for one item.
struct Item {
    int32_t i;
    uint32_t u;
    double d;
};

template <typename T>
T load_le(const unsigned char *p) {
    T v;
    std::memcpy(&v, p, sizeof(T));  // both supported hosts are little-endian
    return v;
}

// A stored float after plyfile's float -> double -> float round trip
// (get_binary_item then store_item): identity, except that a signalling NaN
// comes back quiet with its payload kept (IEEE 754 conversion, as x86 and
// Arm perform it).  Written out so no compiler folds the round trip away.
float float_round_trip(const unsigned char *p) {
    uint32_t u;
    std::memcpy(&u, p, 4);
    if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x007FFFFFu)) u |= 0x00400000u;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// get_binary_item (plyfile.c:2132-2196)
Item binary_item(const unsigned char *p, int type) {
    Item r{};
    switch (type) {
        case kChar: r.i = (int32_t)(int8_t)p[0]; r.u = (uint32_t)r.i; r.d = r.i; break;  // x86 char is signed
        case kUChar: r.u = p[0]; r.i = (int32_t)r.u; r.d = r.u; break;
        case kShort: r.i = load_le<int16_t>(p); r.u = (uint32_t)r.i; r.d = r.i; break;
        case kUShort: r.u = load_le<uint16_t>(p); r.i = (int32_t)r.u; r.d = r.u; break;
        case kInt: r.i = load_le<int32_t>(p); r.u = (uint32_t)r.i; r.d = r.i; break;
        case kUInt: r.u = load_le<uint32_t>(p); r.i = (int32_t)r.u; r.d = r.u; break;
        case kFloat: r.d = load_le<float>(p); r.i = (int32_t)r.d; r.u = (uint32_t)(int64_t)r.d; break;
        case kDouble: r.d = load_le<double>(p); r.i = (int32_t)r.d; r.u = (uint32_t)(int64_t)r.d; break;
        default: break;
    }
    return r;
}

// get_ascii_item (plyfile.c:2212-2247)
Item ascii_item(const char *w, int type) {
    Item r{};
    switch (type) {
        case kChar: case kUChar: case kShort: case kUShort: case kInt:
            r.i = (int32_t)std::strtol(w, nullptr, 10); r.u = (uint32_t)r.i; r.d = r.i; break;
        case kUInt:
            r.u = (uint32_t)std::strtoul(w, nullptr, 10); r.i = (int32_t)r.u; r.d = r.u; break;
        case kFloat: case kDouble:
            r.d = std::strtod(w, nullptr); r.i = (int32_t)r.d; r.u = (uint32_t)(int64_t)r.d; break;
        default: break;
    }
    return r;
}

float swap_f32(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
    std::memcpy(&f, &u, 4);
    return f;
}

int32_t swap_i32(int32_t v) {
    uint32_t u = (uint32_t)v;
    u = (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
    return (int32_t)u;
}

// Whitespace-separated words of one line, as plyfile's get_words splits them.
void split_words(const std::string &line, std::vector<std::string> &out) {
    out.clear();
    size_t i = 0, n = line.size();
    while (i < n) {
        while (i < n && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r' || line[i] == '\n')) ++i;
        size_t j = i;
        while (j < n && !(line[j] == ' ' || line[j] == '\t' || line[j] == '\r' || line[j] == '\n')) ++j;
        if (j > i) out.emplace_back(line.substr(i, j - i));
        i = j;
    }
}

// The file's bytes: mapped read-only (no copy), or read into memory where
// mapping fails.
struct Reader {
    const unsigned char *data = nullptr;
    size_t size = 0, pos = 0;
    void *map = nullptr;
    std::vector<unsigned char> copy;
    ~Reader() {
        if (map) munmap(map, size);
    }
    bool line(std::string &out) {
        if (pos >= size) return false;
        size_t e = pos;
        while (e < size && data[e] != '\n') ++e;
        out.assign((const char *)data + pos, e - pos);
        pos = e < size ? e + 1 : e;
        return true;
    }
};

// Runs fn(begin, end, part) over [0, n) in `parts` contiguous pieces on
// worker threads (inline when there is one part).
template <typename Fn>
void parallel_parts(uint64_t n, int parts, Fn fn) {
    if (parts <= 1) {
        fn((uint64_t)0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    for (int p = 0; p < parts; ++p)
        th.emplace_back([=, &fn] { fn(n * p / parts, n * (p + 1) / parts, p); });
    for (auto &t : th) t.join();
}

int worker_count(uint64_t n) {
    if (n < (1u << 15)) return 1;
    unsigned hw = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(hw ? hw : 1u, 16u));
}

const int kVertexProps = 9;
const char *const kVertexNames[kVertexProps] = {"x", "y", "z", "nx", "ny", "nz", "red", "green", "blue"};

// Float value of one stored binary item, as binary_item(...).d converted to
// float (plyfile's store_item for PLY_FLOAT).
inline float binary_float(const unsigned char *p, int type) {
    switch (type) {
        case kFloat: return float_round_trip(p);
        case kUChar: return (float)p[0];
        case kChar: return (float)(int8_t)p[0];
        case kShort: return (float)load_le<int16_t>(p);
        case kUShort: return (float)load_le<uint16_t>(p);
        case kInt: return (float)(double)load_le<int32_t>(p);
        case kUInt: return (float)(double)load_le<uint32_t>(p);
        case kDouble: return (float)load_le<double>(p);
        default: return 0.0f;
    }
}

// Int value of one stored binary item (binary_item(...).i).
inline int32_t binary_int(const unsigned char *p, int type) {
    switch (type) {
        case kInt: return load_le<int32_t>(p);
        case kUInt: return (int32_t)load_le<uint32_t>(p);
        case kUChar: return p[0];
        case kUShort: return load_le<uint16_t>(p);
        case kShort: return load_le<int16_t>(p);
        case kChar: return (int8_t)p[0];
        default: return binary_item(p, type).i;
    }
}

}  // namespace

void mesh_add_vertex(MeshHost &m, const float p[3], const float *n, const float c[3]) {
    for (int t = 0; t < 3; ++t) {
        m.pos.push_back(p[t]);
        m.col.push_back(c[t]);
        if (n) m.nrm.push_back(n[t]);
        m.lower[t] = (p[t] < m.lower[t]) ? p[t] : m.lower[t];  // std::min(_lower, v)
        m.upper[t] = (m.upper[t] < p[t]) ? p[t] : m.upper[t];  // std::max(_upper, v)
    }
}

int mesh_add_face(MeshHost &m, const int32_t *idx, int count, uint64_t n_vertices) {
    if (count < 3) return SVO_OK;
    for (int k = 0; k < count; ++k)
        if (idx[k] < 0 || (uint64_t)idx[k] >= n_vertices)
            return set_error(SVO_ERR_FORMAT, "PLY face index %d outside the %llu vertices", idx[k],
                             (unsigned long long)n_vertices);
    int32_t v0 = idx[0], v1 = idx[1];
    for (int k = 2; k < count; ++k) {
        m.tris.push_back(v0);
        m.tris.push_back(v1);
        m.tris.push_back(idx[k]);
        v1 = idx[k];
    }
    return SVO_OK;
}

int ply_read(const char *path, MeshHost &out) {
    Reader rd;
    {
        int fd = open(path, O_RDONLY);
        if (fd < 0) return set_error(SVO_ERR_IO, "cannot open PLY %s: %s", path, std::strerror(errno));
        struct stat stt;
        if (fstat(fd, &stt) != 0) {
            close(fd);
            return set_error(SVO_ERR_IO, "cannot size PLY %s", path);
        }
        rd.size = (size_t)stt.st_size;
        if (rd.size) {
            void *mp = mmap(nullptr, rd.size, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
            if (mp != MAP_FAILED) {
                rd.map = mp;
                rd.data = (const unsigned char *)mp;
            } else {
                rd.copy.resize(rd.size);
                size_t got = 0;
                while (got < rd.size) {
                    ssize_t r = read(fd, rd.copy.data() + got, rd.size - got);
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got != rd.size) {
                    close(fd);
                    return set_error(SVO_ERR_IO, "short read on PLY %s", path);
                }
                rd.data = rd.copy.data();
            }
        }
        close(fd);
    }

    // Header (plyfile.c ply_read, :700-790).
    std::string line;
    std::vector<std::string> w;
    if (!rd.line(line)) return set_error(SVO_ERR_FORMAT, "%s: empty file", path);
    split_words(line, w);
    if (w.size() != 1 || w[0] != "ply") return set_error(SVO_ERR_FORMAT, "%s: not a PLY file", path);
    int format = -1;  // 0 ascii, 1 binary LE, 2 binary BE
    std::vector<Elem> elems;
    bool header_done = false;
    while (rd.line(line)) {
        split_words(line, w);
        if (w.empty()) continue;
        if (w[0] == "format" && w.size() >= 2) {
            if (w[1] == "ascii") format = 0;
            else if (w[1] == "binary_little_endian") format = 1;
            else if (w[1] == "binary_big_endian") format = 2;
            else return set_error(SVO_ERR_FORMAT, "%s: unknown PLY format %s", path, w[1].c_str());
        } else if (w[0] == "element" && w.size() >= 3) {
            Elem e;
            e.name = w[1];
            e.count = std::strtoull(w[2].c_str(), nullptr, 10);
            elems.push_back(e);
        } else if (w[0] == "property" && w.size() >= 3) {
            if (elems.empty()) return set_error(SVO_ERR_FORMAT, "%s: property before any element", path);
            Prop p;
            if (w[1] == "list") {
                if (w.size() < 5) return set_error(SVO_ERR_FORMAT, "%s: bad list property", path);
                p.count_type = parse_type(w[2]);
                p.type = parse_type(w[3]);
                p.name = w[4];
                if (p.count_type == kInvalid || p.type == kInvalid)
                    return set_error(SVO_ERR_FORMAT, "%s: bad list property types", path);
            } else {
                p.type = parse_type(w[1]);
                p.name = w[2];
                if (p.type == kInvalid) return set_error(SVO_ERR_FORMAT, "%s: bad property type %s", path, w[1].c_str());
            }
            elems.back().props.push_back(p);
        } else if (w[0] == "end_header") {
            header_done = true;
            break;
        }
    }
    if (!header_done || format < 0) return set_error(SVO_ERR_FORMAT, "%s: incomplete PLY header", path);
    const Elem *ve = nullptr, *fe = nullptr;
    for (const Elem &e : elems) {
        if (e.name == "vertex" && !ve) ve = &e;
        else if (e.name == "face" && !fe) fe = &e;
    }
    if (!ve || !fe) return set_error(SVO_ERR_FORMAT, "%s: PLY file has to have triangles and vertices", path);

    // Vertex property slots (PlyLoader.cpp:128-142) and the face index list.
    int vslot[64];
    bool avail[kVertexProps] = {};
    if (ve->props.size() > 64) return set_error(SVO_ERR_LIMIT, "%s: more than 64 vertex properties", path);
    for (size_t i = 0; i < ve->props.size(); ++i) {
        vslot[i] = -1;
        for (int t = 0; t < kVertexProps; ++t)
            if (ve->props[i].name == kVertexNames[t]) {
                vslot[i] = t;
                avail[t] = true;
                break;
            }
    }
    int face_prop = -1;
    for (size_t i = 0; i < fe->props.size(); ++i)
        if (fe->props[i].name == "vertex_indices") {
            face_prop = (int)i;
            break;
        }
    if (face_prop < 0 || fe->props[face_prop].count_type == kInvalid)
        return set_error(SVO_ERR_FORMAT, "%s: no face information found", path);
    const bool has_normals = avail[3] && avail[4] && avail[5];
    const bool be = format == 2;

    out = MeshHost();
    out.pos.reserve(ve->count * 3);
    out.col.reserve(ve->count * 3);
    if (has_normals) out.nrm.reserve(ve->count * 3);
    out.tris.reserve(fe->count * 3);

    const float vdefault[kVertexProps] = {0, 0, 0, 0, 0, 0, 255.0f, 255.0f, 255.0f};
    std::vector<int32_t> idx;
    for (const Elem &e : elems) {
        const bool is_v = &e == ve, is_f = &e == fe;
        bool scalar_only = true;
        size_t stride = 0;
        for (const Prop &p : e.props) {
            if (p.count_type != kInvalid) scalar_only = false;
            else stride += type_size(p.type);
        }
        if (format != 0 && is_v && scalar_only) {
            // Fixed-size vertex records: convert the wanted properties in place.
            if (rd.pos + stride * e.count > rd.size) return set_error(SVO_ERR_FORMAT, "%s: truncated PLY", path);
            int off[kVertexProps], typ[kVertexProps];
            for (int t = 0; t < kVertexProps; ++t) off[t] = -1, typ[t] = kInvalid;
            size_t o = 0;
            for (size_t pi = 0; pi < e.props.size(); ++pi) {
                if (vslot[pi] >= 0) {
                    off[vslot[pi]] = (int)o;
                    typ[vslot[pi]] = e.props[pi].type;
                }
                o += type_size(e.props[pi].type);
            }
            const uint64_t n = e.count;
            out.pos.resize(n * 3);
            out.col.resize(n * 3);
            if (has_normals) out.nrm.resize(n * 3);
            const unsigned char *base0 = rd.data + rd.pos;
            const int parts = worker_count(n);
            // per-part bounds, folded in part order afterwards: std::min keeps
            // the first of equal values, and so does this in-order fold
            std::vector<float> plo(3 * parts, 1e30f), phi(3 * parts, -1e30f);
            std::atomic<uint64_t> bad{~0ull};
            parallel_parts(n, parts, [&](uint64_t b, uint64_t e_, int part) {
                float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
                const unsigned char *base = base0 + b * stride;
                for (uint64_t k = b; k < e_; ++k, base += stride) {
                    float vd[kVertexProps];
                    for (int t = 0; t < kVertexProps; ++t) {
                        if (off[t] < 0) {
                            vd[t] = vdefault[t];
                        } else {
                            float f = binary_float(base + off[t], typ[t]);
                            vd[t] = be ? swap_f32(f) : f;
                        }
                    }
                    for (int t = 0; t < 3; ++t) {
                        if (!std::isfinite(vd[t])) {
                            uint64_t cur = bad.load();
                            while (k < cur && !bad.compare_exchange_weak(cur, k)) {
                            }
                        }
                        out.pos[3 * k + t] = vd[t];
                        out.col[3 * k + t] = vd[6 + t];
                        if (has_normals) out.nrm[3 * k + t] = vd[3 + t];
                        lo[t] = (vd[t] < lo[t]) ? vd[t] : lo[t];
                        hi[t] = (hi[t] < vd[t]) ? vd[t] : hi[t];
                    }
                }
                for (int t = 0; t < 3; ++t) {
                    plo[3 * part + t] = lo[t];
                    phi[3 * part + t] = hi[t];
                }
            });
            if (bad.load() != ~0ull)
                return set_error(SVO_ERR_FORMAT, "%s: vertex %llu has a non-finite coordinate", path,
                                 (unsigned long long)bad.load());
            for (int part = 0; part < parts; ++part)
                for (int t = 0; t < 3; ++t) {
                    float l = plo[3 * part + t], h = phi[3 * part + t];
                    out.lower[t] = (l < out.lower[t]) ? l : out.lower[t];
                    out.upper[t] = (out.upper[t] < h) ? h : out.upper[t];
                }
            rd.pos += stride * e.count;
            continue;
        }
        if (format != 0 && is_f) {
            // Faces: scalars skipped by size, the index list read directly.
            const Prop &lp = e.props[face_prop];
            const int cs = type_size(lp.count_type), is = type_size(lp.type);
            size_t pre = 0, post = 0;
            bool simple = true;
            for (size_t pi = 0; pi < e.props.size(); ++pi) {
                if ((int)pi == face_prop) continue;
                if (e.props[pi].count_type != kInvalid) simple = false;
                else if ((int)pi < face_prop) pre += type_size(e.props[pi].type);
                else post += type_size(e.props[pi].type);
            }
            if (simple && e.count > 0) {
                // All faces triangles (checked face by face): fixed-size
                // records, converted in parallel.
                const uint64_t nv = ve->count;
                const size_t rec = pre + cs + 3 * (size_t)is + post;
                if (rd.pos + rec * e.count <= rd.size) {
                    const unsigned char *base0 = rd.data + rd.pos;
                    const uint64_t n = e.count;
                    const size_t t0 = out.tris.size();
                    out.tris.resize(t0 + 3 * n);
                    std::atomic<bool> uniform{true};
                    std::atomic<uint64_t> bad{~0ull};
                    parallel_parts(n, worker_count(n), [&](uint64_t b, uint64_t e_, int) {
                        const unsigned char *r = base0 + b * rec;
                        for (uint64_t k = b; k < e_; ++k, r += rec) {
                            if (binary_int(r + pre, lp.count_type) != 3) {
                                uniform.store(false);
                                return;
                            }
                            for (int c = 0; c < 3; ++c) {
                                int32_t x = binary_int(r + pre + cs + (size_t)c * is, lp.type);
                                x = be ? swap_i32(x) : x;
                                if (x < 0 || (uint64_t)x >= nv) bad.store(k);
                                out.tris[t0 + 3 * k + c] = x;
                            }
                        }
                    });
                    if (uniform.load()) {
                        if (bad.load() != ~0ull)
                            return set_error(SVO_ERR_FORMAT, "%s: face %llu has an index outside the %llu vertices",
                                             path, (unsigned long long)bad.load(), (unsigned long long)nv);
                        rd.pos += rec * e.count;
                        continue;
                    }
                    out.tris.resize(t0);
                }
            }
            if (simple) {
                const uint64_t nv = ve->count;
                const unsigned char *buf = rd.data;
                const size_t size = rd.size;
                size_t pos = rd.pos;
                int32_t ib[256];
                for (uint64_t k = 0; k < e.count; ++k) {
                    if (pos + pre + cs > size) return set_error(SVO_ERR_FORMAT, "%s: truncated PLY", path);
                    pos += pre;
                    int cnt = binary_int(buf + pos, lp.count_type);
                    pos += cs;
                    if (cnt < 0 || pos + (size_t)cnt * is + post > size)
                        return set_error(SVO_ERR_FORMAT, "%s: truncated PLY list", path);
                    if (cnt >= 3) {
                        int32_t *v = cnt <= 256 ? ib : nullptr;
                        std::vector<int32_t> big;
                        if (!v) {
                            big.resize(cnt);
                            v = big.data();
                        }
                        for (int c = 0; c < cnt; ++c) {
                            int32_t x = binary_int(buf + pos + (size_t)c * is, lp.type);
                            v[c] = be ? swap_i32(x) : x;
                            if (v[c] < 0 || (uint64_t)v[c] >= nv)
                                return set_error(SVO_ERR_FORMAT, "PLY face index %d outside the %llu vertices", v[c],
                                                 (unsigned long long)nv);
                        }
                        for (int c = 2; c < cnt; ++c) {  // PlyLoader.cpp:208-220
                            out.tris.push_back(v[0]);
                            out.tris.push_back(c == 2 ? v[1] : v[c - 1]);
                            out.tris.push_back(v[c]);
                        }
                    }
                    pos += (size_t)cnt * is + post;
                }
                rd.pos = pos;
                continue;
            }
        }
        for (uint64_t k = 0; k < e.count; ++k) {
            float vd[kVertexProps];
            for (int t = 0; t < kVertexProps; ++t) vd[t] = vdefault[t];
            idx.clear();
            if (format == 0) {
                if (!rd.line(line)) return set_error(SVO_ERR_FORMAT, "%s: truncated ascii PLY", path);
                split_words(line, w);
                size_t wi = 0;
                for (size_t pi = 0; pi < e.props.size(); ++pi) {
                    const Prop &p = e.props[pi];
                    if (p.count_type != kInvalid) {
                        if (wi >= w.size()) return set_error(SVO_ERR_FORMAT, "%s: short ascii PLY line", path);
                        int cnt = ascii_item(w[wi++].c_str(), p.count_type).i;
                        if (cnt < 0 || wi + (size_t)cnt > w.size())
                            return set_error(SVO_ERR_FORMAT, "%s: short ascii PLY list", path);
                        for (int c = 0; c < cnt; ++c) {
                            Item it = ascii_item(w[wi++].c_str(), p.type);
                            if (is_f && (int)pi == face_prop) idx.push_back(it.i);
                        }
                    } else {
                        if (wi >= w.size()) return set_error(SVO_ERR_FORMAT, "%s: short ascii PLY line", path);
                        Item it = ascii_item(w[wi++].c_str(), p.type);
                        if (is_v && vslot[pi] >= 0) vd[vslot[pi]] = (float)it.d;
                    }
                }
            } else {
                for (size_t pi = 0; pi < e.props.size(); ++pi) {
                    const Prop &p = e.props[pi];
                    if (p.count_type != kInvalid) {
                        int cs = type_size(p.count_type), is = type_size(p.type);
                        if (rd.pos + cs > rd.size) return set_error(SVO_ERR_FORMAT, "%s: truncated PLY", path);
                        int cnt = binary_item(rd.data + rd.pos, p.count_type).i;
                        rd.pos += cs;
                        if (cnt < 0 || rd.pos + (size_t)cnt * is > rd.size)
                            return set_error(SVO_ERR_FORMAT, "%s: truncated PLY list", path);
                        for (int c = 0; c < cnt; ++c) {
                            if (is_f && (int)pi == face_prop) {
                                int32_t v = binary_item(rd.data + rd.pos, p.type).i;
                                idx.push_back(be ? swap_i32(v) : v);
                            }
                            rd.pos += is;
                        }
                    } else {
                        int is = type_size(p.type);
                        if (rd.pos + is > rd.size) return set_error(SVO_ERR_FORMAT, "%s: truncated PLY", path);
                        if (is_v && vslot[pi] >= 0) {
                            float f = binary_float(rd.data + rd.pos, p.type);
                            vd[vslot[pi]] = be ? swap_f32(f) : f;
                        }
                        rd.pos += is;
                    }
                }
            }
            if (is_v) {
                for (int t = 0; t < 3; ++t)
                    if (!std::isfinite(vd[t]))
                        return set_error(SVO_ERR_FORMAT, "%s: vertex %llu has a non-finite coordinate", path,
                                         (unsigned long long)k);
                mesh_add_vertex(out, vd, has_normals ? vd + 3 : nullptr, vd + 6);
            } else if (is_f) {
                int rc = mesh_add_face(out, idx.data(), (int)idx.size(), ve->count);
                if (rc) return rc;
            }
        }
    }
    return SVO_OK;
}

}  // namespace svo
