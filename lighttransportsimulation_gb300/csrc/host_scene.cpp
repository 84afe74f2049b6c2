// Host loader for the reference's input files.  Compiled with -ffp-contract=off so that
// every float expression below rounds exactly as the reference's host code does
// (core/SceneLoader.cuh, core/FileIO.cuh, geometry/Transform.cuh, rendering/Camera.cu,
// rendering/Filter.cuh, intergrators/IntegratorHelper.cuh, sampling/Sampling.cuh).
#include "host_scene.hpp"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <stdexcept>
#include <algorithm>
#include <atomic>
#include <sstream>
#include <thread>
#include <utility>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/lts_capi.h"

namespace lts {
namespace {

// M_PI as <math.h> defines it on Linux (a double): the reference's `#ifndef M_PI` fallback
// (core/GeneralHelper.cuh:8-10) is not taken there.
constexpr double kPi = 3.14159265358979323846;

struct V3 {
    float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(V3 a, float f) { return {f * a.x, f * a.y, f * a.z}; }  // Vector3::operator*(U f): f * x
inline float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// geometry/Geometry.cuh:76-83: products and differences in double, rounded to float once.
inline V3 cross_d(V3 a, V3 b) {
    const double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return {(float)((ay * bz) - (az * by)), (float)((az * bx) - (ax * bz)), (float)((ax * by) - (ay * bx))};
}
inline V3 normalize_q(V3 v) { return scale(v, quake_rsqrt(len2(v))); }

struct Quat {
    float w = 1, x = 0, y = 0, z = 0;
};
// geometry/Transform.cuh:71-80 (quaternionMult), left-to-right sums.
inline Quat qmul(const Quat& a, const Quat& b) {
    Quat r;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
    r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
    return r;
}
inline Quat conj(const Quat& q) { return Quat{q.w, -q.x, -q.y, -q.z}; }

struct Xform {  // geometry/Transform.cuh:138-200 (translation, rotation, scale)
    V3 t{0, 0, 0};
    Quat r;
    float s = 1;
    // Point/vector transform, Transform.cuh:222-233: rotate, scale, translate.
    V3 point(V3 p) const {
        Quat q{0.0f, p.x, p.y, p.z};
        Quat tq = qmul(qmul(r, q), conj(r));
        return add(scale(V3{tq.x, tq.y, tq.z}, s), t);
    }
    // Normal transform, Transform.cuh:235-240: inverse rotation, then normalize.
    V3 normal(V3 n) const {
        Quat q{0.0f, n.x, n.y, n.z};
        Quat tq = qmul(qmul(conj(r), q), r);
        return normalize_q(V3{tq.x, tq.y, tq.z});
    }
};

Xform make_xform(V3 t, V3 axis, float theta, float scl) {
    Xform x;
    x.t = t;
    const float th = fmodf(theta, (float)(2 * kPi));  // Transform.cuh:170-175
    x.r.w = cosf(th / 2);                              // axisAngleToQuaternion, :109-115
    x.r.x = axis.x * sinf(th / 2);
    x.r.y = axis.y * sinf(th / 2);
    x.r.z = axis.z * sinf(th / 2);
    x.s = scl;
    return x;
}

class Tokens {
   public:
    bool open(const std::string& path) {
        std::ifstream f(path);
        if (!f.is_open()) return false;
        std::stringstream ss;
        ss << f.rdbuf();
        data_ = ss.str();
        return true;
    }
    bool next(std::string* t) {
        while (pos_ < data_.size() && isspace((unsigned char)data_[pos_])) ++pos_;
        if (pos_ >= data_.size()) return false;
        size_t b = pos_;
        while (pos_ < data_.size() && !isspace((unsigned char)data_[pos_])) ++pos_;
        *t = data_.substr(b, pos_ - b);
        return true;
    }

   private:
    std::string data_;
    size_t pos_ = 0;
};

// f(begin, end) over [0, n) in contiguous chunks on up to 16 host threads (serially below 32K
// items).  The loops it runs write disjoint elements, so the result does not depend on the split.
template <class F>
void parallel_ranges(size_t n, const F& f) {
    const size_t kMin = size_t(1) << 15;
    unsigned nt = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (n < 2 * kMin || nt <= 1) {
        f(size_t(0), n);
        return;
    }
    nt = (unsigned)std::min<size_t>(nt, n / kMin);
    const size_t chunk = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (unsigned k = 1; k < nt; ++k) {
        const size_t b = k * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
    }
    f(size_t(0), std::min(n, chunk));
    for (auto& t : th) t.join();
}

struct ParseError {
    int code;
    std::string msg;
};

std::string tok(Tokens& s, const char* what) {
    std::string t;
    if (!s.next(&t)) throw ParseError{LTS_ERR_PARSE, std::string("unexpected end of file reading ") + what};
    return t;
}
float tokf(Tokens& s, const char* what) {
    std::string t = tok(s, what);
    try {
        return std::stof(t);
    } catch (...) {
        throw ParseError{LTS_ERR_PARSE, std::string("bad number '") + t + "' for " + what};
    }
}
int toki(Tokens& s, const char* what) {
    std::string t = tok(s, what);
    try {
        return std::stoi(t);
    } catch (...) {
        throw ParseError{LTS_ERR_PARSE, std::string("bad integer '") + t + "' for " + what};
    }
}

// One mesh file: the whole .bin image (read_bin) or the vectors parse_obj fills; P(), UV(), N()
// and I() view either.
struct MeshData {
    int32_t ntri = 0, np = 0, nuv = 0, nn = 0;
    HostVec<char> bin;                  // .bin file: 16-byte header, P, UV, N, indices
    std::vector<float> sp, suv, sn;     // .obj
    std::vector<int32_t> sidx;
    const float* P() const { return bin.empty() ? sp.data() : reinterpret_cast<const float*>(bin.data() + 16); }
    const float* UV() const { return bin.empty() ? suv.data() : P() + 3 * (size_t)np; }
    const float* N() const { return bin.empty() ? sn.data() : UV() + 2 * (size_t)nuv; }
    const int32_t* I() const {
        return bin.empty() ? sidx.data() : reinterpret_cast<const int32_t*>(N() + 3 * (size_t)nn);
    }
};

// core/FileIO.cuh:170-206 (binMeshRead), with size checks the reference does not make.  The file
// is read whole, in contiguous parts on up to 16 threads (positioned reads), into a buffer that is
// not zeroed first.
MeshData read_bin(const std::string& path) {
    const int fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) throw ParseError{LTS_ERR_IO, "cannot open mesh " + path};
    struct stat st;
    if (::fstat(fd, &st) != 0) {
        ::close(fd);
        throw ParseError{LTS_ERR_IO, "cannot stat mesh " + path};
    }
    const long long size = (long long)st.st_size;
    MeshData m;
    m.bin.resize((size_t)std::max(0LL, size));
    std::atomic<bool> failed{false};
    parallel_ranges((size_t)m.bin.size(), [&](size_t b, size_t e) {
        while (b < e) {
            const ssize_t r = ::pread(fd, m.bin.data() + b, e - b, (off_t)b);
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) {
                failed = true;
                return;
            }
            b += (size_t)r;
        }
    });
    ::close(fd);
    if (failed) throw ParseError{LTS_ERR_IO, "cannot read mesh " + path};
    int32_t hdr[4];
    if (size < 16) throw ParseError{LTS_ERR_PARSE, "short mesh header in " + path};
    std::memcpy(hdr, m.bin.data(), 16);
    m.ntri = hdr[0];
    m.np = hdr[1];
    m.nuv = hdr[2];
    m.nn = hdr[3];
    if (m.ntri < 0 || m.np < 0 || m.nuv < 0 || m.nn < 0)
        throw ParseError{LTS_ERR_PARSE, "negative counts in " + path};
    const long long need = 16 + 12LL * m.np + 8LL * m.nuv + 12LL * m.nn + 36LL * m.ntri;
    if (size < need) throw ParseError{LTS_ERR_PARSE, "truncated mesh " + path};
    return m;
}

// Every corner's position index, and its uv / normal index when the mesh has any, in range (the
// reference reads out of bounds otherwise).
void check_indices(const MeshData& m, const std::string& name) {
    std::atomic<bool> bad{false};
    const int32_t* idx = m.I();
    parallel_ranges((size_t)m.ntri, [&](size_t b, size_t e) {
        for (size_t t = b; t < e; ++t)
            for (int c = 0; c < 3; ++c) {
                const int32_t ip = idx[9 * t + 3 * c], iu = idx[9 * t + 3 * c + 1], in = idx[9 * t + 3 * c + 2];
                if (ip < 0 || ip >= m.np || (m.nuv > 0 && (iu < 0 || iu >= m.nuv)) ||
                    (m.nn > 0 && (in < 0 || in >= m.nn))) {
                    bad = true;
                    return;
                }
            }
    });
    if (bad) throw ParseError{LTS_ERR_PARSE, "vertex index out of range in mesh " + name};
}

// core/FileIO.cuh:73-164 (parseMeshFile): the whole file is read as whitespace-separated tokens
// (no comment handling: a token of a comment or of an unknown statement is skipped like any other
// token, so a "v" inside a comment still reads a vertex); "v" / "vn" take the next three tokens
// and "vt" the next two as floats (std::stof: leading number of the token); "f" takes the next
// three tokens as "p/uv/n" 1-based indices.  The uv index is read only once some "vt" has been
// seen (0 before); an index field that does not start with a number keeps the value read last in
// the same face corner (std::from_chars leaves its output unchanged on failure).  Where the
// reference's behaviour is undefined (no number at all before the first field, fewer than three
// fields, a token that stof rejects, missing tokens at the end) this reader raises a parse error.
MeshData parse_obj(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f.good()) throw ParseError{LTS_ERR_IO, "cannot open mesh " + path + " (neither .bin nor .obj)"};
    std::ostringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    size_t pos = 0;
    auto next = [&](std::string& t) -> bool {  // operator>>(istream&, string&)
        while (pos < text.size() && std::isspace((unsigned char)text[pos])) ++pos;
        if (pos >= text.size()) return false;
        const size_t b = pos;
        while (pos < text.size() && !std::isspace((unsigned char)text[pos])) ++pos;
        t.assign(text, b, pos - b);
        return true;
    };
    auto num = [&](const char* what) -> float {
        std::string t;
        if (!next(t)) throw ParseError{LTS_ERR_PARSE, std::string("missing ") + what + " in " + path};
        errno = 0;
        char* end = nullptr;
        const float v = std::strtof(t.c_str(), &end);
        if (end == t.c_str() || errno == ERANGE)  // std::stof throws on both
            throw ParseError{LTS_ERR_PARSE, "bad number '" + t + "' for " + what + " in " + path};
        return v;
    };
    // std::from_chars(int) over [b, e): leading digits with an optional '-'; false leaves i as is
    auto field = [](const char* b, const char* e, int& i) -> bool {
        const char* q = b;
        bool neg = false;
        if (q < e && *q == '-') {
            neg = true;
            ++q;
        }
        if (q >= e || *q < '0' || *q > '9') return false;
        long long v = 0;
        for (; q < e && *q >= '0' && *q <= '9'; ++q) {
            v = v * 10 + (*q - '0');
            if (v > 2147483648LL) return false;  // out of range: from_chars reports an error
        }
        v = neg ? -v : v;
        if (v > 2147483647LL || v < -2147483648LL) return false;
        i = (int)v;
        return true;
    };
    MeshData m;
    std::string t;
    while (next(t)) {
        if (t == "v") {
            for (int k = 0; k < 3; ++k) m.sp.push_back(num("vertex"));
        } else if (t == "vt") {
            for (int k = 0; k < 2; ++k) m.suv.push_back(num("texture coordinate"));
        } else if (t == "vn") {
            for (int k = 0; k < 3; ++k) m.sn.push_back(num("normal"));
        } else if (t == "f") {
            for (int c = 0; c < 3; ++c) {
                std::string corner;
                if (!next(corner)) throw ParseError{LTS_ERR_PARSE, "missing face corner in " + path};
                std::vector<std::pair<size_t, size_t>> parts;  // FileIO.cuh:50-66 split on '/'
                size_t b = 0;
                for (;;) {
                    const size_t e = corner.find('/', b);
                    parts.emplace_back(b, (e == std::string::npos ? corner.size() : e) - b);
                    if (e == std::string::npos) break;
                    b = e + 1;
                }
                const bool with_uv = !m.suv.empty();
                if (parts.size() < 3)
                    throw ParseError{LTS_ERR_PARSE, "face corner '" + corner + "' is not p/uv/n in " + path};
                const char* base = corner.data();
                int i = 0;
                if (!field(base + parts[0].first, base + parts[0].first + parts[0].second, i))
                    throw ParseError{LTS_ERR_PARSE, "face corner '" + corner + "' has no vertex index in " + path};
                m.sidx.push_back(i - 1);
                if (with_uv) {
                    field(base + parts[1].first, base + parts[1].first + parts[1].second, i);
                    m.sidx.push_back(i - 1);
                } else {
                    m.sidx.push_back(0);
                }
                field(base + parts[2].first, base + parts[2].first + parts[2].second, i);
                m.sidx.push_back(i - 1);
            }
            ++m.ntri;
        }
    }
    m.np = (int32_t)(m.sp.size() / 3);
    m.nuv = (int32_t)(m.suv.size() / 2);
    m.nn = (int32_t)(m.sn.size() / 3);
    return m;
}

// core/FileIO.cuh:20-45 (binMeshWrite): header nTri nP nUV nN, then P, UV, N, indices.
bool write_bin(const std::string& path, const MeshData& m) {
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f.good()) return false;
    const int32_t hdr[4] = {m.ntri, m.np, m.nuv, m.nn};
    f.write((const char*)hdr, 16);
    f.write((const char*)m.P(), 12LL * m.np);
    f.write((const char*)m.UV(), 8LL * m.nuv);
    f.write((const char*)m.N(), 12LL * m.nn);
    f.write((const char*)m.I(), 36LL * m.ntri);
    return f.good();
}

// core/FileIO.cuh:213-232 (parseMesh): meshName.bin when it opens, else meshName.obj, whose
// conversion is also written to meshName.bin (as the reference does; a failed write is ignored).
MeshData read_mesh(const std::string& name) {
    {
        std::ifstream probe(name + ".bin", std::ios::binary);
        if (probe.good()) return read_bin(name + ".bin");
    }
    MeshData m = parse_obj(name + ".obj");
    write_bin(name + ".bin", m);
    return m;
}

HostTexture read_texture(Tokens& s, bool scene_stream, int subject_images) {
    HostTexture t;
    const std::string ty = tok(s, "texture type");
    const char c = ty[0];
    int len = 0;  // SceneLoader.cuh:147-150
    if (c == 'i') len = 1;
    else if (c == 'f' || c == 'w') len = 2;
    else if (c == 'c') len = 3;
    else if (c == 'm') len = 4;
    float v[4] = {0, 0, 0, 0};
    for (int i = 0; i < len; ++i) {
        v[i] = tokf(s, "texture parameter");
        if (c == 'i' && scene_stream) v[i] += subject_images;
    }
    switch (c) {  // setMatTexture, SceneLoader.cuh:362-391
        case 'c': t.kind = TEX_CONSTANT; break;
        case 'f': t.kind = TEX_FBM; break;
        case 'w': t.kind = TEX_WRINKLED; break;
        case 'm': t.kind = TEX_MARBLE; break;
        case 'v': t.kind = TEX_WINDY; break;
        case 'i': t.kind = TEX_IMAGE; break;  // ImageTexture over mipmap v[0], UV mapping (1, 1, 0, 0)
        default:
            throw ParseError{LTS_ERR_UNSUPPORTED, std::string("texture type '") + c + "' is not supported"};
    }
    memcpy(t.v, v, sizeof v);
    return t;
}

}  // namespace

// Camera (rendering/Camera.cu:9-43) with aperture 0 (LightTransportSimulation.cu:70) from the
// scene file's camera record cf = from(3), at(3), up(3), vfov (degrees), focus distance.
void build_camera(const float cf[11], int width, int height, float cam[23]) {
    const V3 from{cf[0], cf[1], cf[2]}, at{cf[3], cf[4], cf[5]}, vup{cf[6], cf[7], cf[8]};
    const float vfov = cf[9], focus = cf[10];
    const float aspect = (float)width / (float)height;
    const float theta = (float)((double)vfov * kPi / 180.0f);
    const float h = tanf(theta / 2);
    const float vh = 2 * h, vw = aspect * vh;
    const V3 w = normalize_q(sub(from, at));
    const V3 u = normalize_q(cross_d(vup, w));
    const V3 v = cross_d(w, u);
    const V3 right = scale(u, focus * vw), up = scale(v, focus * vh);
    const V3 llc = sub(sub(sub(from, scale(right, 0.5f)), scale(up, 0.5f)), scale(w, focus));
    const float camv[23] = {from.x, from.y, from.z, right.x, right.y, right.z, up.x, up.y, up.z,
                            llc.x,  llc.y,  llc.z,  u.x,     u.y,     u.z,     v.x,  v.y,  v.z,
                            w.x,    w.y,    w.z,    0.0f / 2, focus};
    memcpy(cam, camv, sizeof camv);
}

// geometry/Geometry.cuh:15-29 with the 32-bit integer read of the Windows (LLP64) build.
float quake_rsqrt(float f) {
    const float threehalfs = 1.5f;
    float x2 = f * 0.5f, y = f;
    int32_t i;
    memcpy(&i, &y, 4);
    i = 0x5f3759df - (i >> 1);
    memcpy(&y, &i, 4);
    y = y * (threehalfs - (x2 * y * y));
    y = y * (threehalfs - (x2 * y * y));
    return y;
}

int32_t HostScene::max_mesh_triangles() const {
    int32_t m = 0;
    for (int32_t c : mesh_tri_count) m = c > m ? c : m;
    return m;
}

void HostScene::triangle_soup(std::vector<float>& out) const {
    const int32_t nt = triangles();
    out.resize(9 * (size_t)nt);
    for (int32_t t = 0; t < nt; ++t)
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) out[9 * (size_t)t + 3 * c + k] = p[3 * (size_t)tri_p[3 * t + c] + k];
}

std::string obj_to_bin(const std::string& mesh_name, int* code) {
    try {
        const MeshData m = parse_obj(mesh_name + ".obj");
        if (!write_bin(mesh_name + ".bin", m)) {
            *code = LTS_ERR_IO;
            return "cannot write " + mesh_name + ".bin";
        }
    } catch (const ParseError& e) {
        *code = e.code;
        return e.msg;
    } catch (const std::bad_alloc&) {
        *code = LTS_ERR_OOM;
        return "out of host memory";
    } catch (const std::exception& e) {  // e.g. std::system_error when a loader thread cannot start
        *code = LTS_ERR_IO;
        return std::string("load failed: ") + e.what();
    }
    *code = LTS_OK;
    return "";
}

std::string read_app_params(const std::string& path, AppParams* out, int* code) {
    Tokens s;
    if (!s.open(path)) {
        *code = LTS_ERR_IO;
        return "cannot open " + path;
    }
    try {  // core/FileIO.cuh:234-257
        out->width = toki(s, "width");
        out->height = toki(s, "height");
        out->spp = toki(s, "spp");
        out->max_bounce = toki(s, "bounces");
        out->rr_start = toki(s, "roulette start");
        out->format = toki(s, "format");
        out->output = tok(s, "output") + (out->format ? ".pfm" : ".hdr");
        out->scene = tok(s, "scene");
        std::string sub;
        out->subject = s.next(&sub) ? sub : "";
    } catch (const ParseError& e) {
        *code = e.code;
        return e.msg;
    } catch (const std::bad_alloc&) {
        *code = LTS_ERR_OOM;
        return "out of host memory";
    } catch (const std::exception& e) {  // e.g. std::system_error when a loader thread cannot start
        *code = LTS_ERR_IO;
        return std::string("load failed: ") + e.what();
    }
    *code = LTS_OK;
    return "";
}

std::string load_scene(const std::string& root, const std::string& scene_name, const std::string& subject_name,
                       int32_t width, int32_t height, HostScene* sc, int* code) {
    *code = LTS_OK;
    if (width < 2 || height < 2) {
        *code = LTS_ERR_ARG;
        return "film must be at least 2x2 (the camera divides by resolution - 1)";
    }
    const bool has_subject = !subject_name.empty();
    Tokens ss, sb;
    if (!ss.open(root + scene_name + ".scene")) {
        *code = LTS_ERR_IO;
        return "cannot open " + root + scene_name + ".scene";
    }
    if (has_subject && !sb.open(root + subject_name + ".subject")) {
        *code = LTS_ERR_IO;
        return "cannot open " + root + subject_name + ".subject";
    }
    try {
        // Camera (SceneLoader.cuh:33-57).
        float cf[11];
        for (int i = 0; i < 11; ++i) cf[i] = tokf(ss, "camera");
        // Subject transform (SceneLoader.cuh:59-77).
        float xf[8];
        for (int i = 0; i < 8; ++i) xf[i] = tokf(ss, "subject transform");
        const Xform subject_xf = make_xform({xf[0], xf[1], xf[2]}, {xf[3], xf[4], xf[5]}, xf[6], xf[7]);

        // Images (SceneLoader.cuh:79-97): wrap mode clamped to 0..2, file under the root; each
        // decoded and given its pyramid (image_io.cpp).
        int sub_images = 0, images = 0;
        if (has_subject) images = sub_images = toki(sb, "subject image count");
        images += toki(ss, "scene image count");
        if (images < 0) throw ParseError{LTS_ERR_PARSE, "negative image count"};
        sc->images.clear();
        sc->images.resize((size_t)images);
        for (int i = 0; i < images; ++i) {
            Tokens& s = i >= sub_images ? ss : sb;
            const int wrap = std::min(2, std::max(0, toki(s, "image wrap")));
            const std::string path = root + tok(s, "image path");
            int w = 0, h = 0, icode = 0;
            std::vector<uint8_t> rgb8;
            const std::string ie = decode_image_file(path, &w, &h, &rgb8, &icode);
            if (!ie.empty()) throw ParseError{icode, ie};
            build_pyramid(w, h, rgb8, wrap, &sc->images[(size_t)i]);
        }
        // Meshes (SceneLoader.cuh:99-113).
        int sub_meshes = 0, meshes = 0;
        if (has_subject) meshes = sub_meshes = toki(sb, "subject mesh count");
        meshes += toki(ss, "scene mesh count");
        std::vector<std::string> files;
        for (int m = 0; m < meshes; ++m) files.push_back(root + tok(m >= sub_meshes ? ss : sb, "mesh path"));
        // Materials (SceneLoader.cuh:115-171; codes of SceneLoader_kernels.cu:8-50).
        int sub_mats = 0, mats = 0;
        if (has_subject) mats = sub_mats = toki(sb, "subject material count");
        mats += toki(ss, "scene material count");
        sc->materials.clear();
        for (int m = 0; m < mats; ++m) {
            const bool scene_stream = m >= sub_mats;
            Tokens& s = scene_stream ? ss : sb;
            const std::string ty = tok(s, "material type");
            HostMaterial hm;
            switch (ty[0]) {
                case 'L': hm.kind = MAT_MATTE; hm.tex[0] = read_texture(s, scene_stream, sub_images); break;
                case 'R': hm.kind = MAT_MIRROR; hm.tex[0] = read_texture(s, scene_stream, sub_images); break;
                case 'G':
                    hm.kind = MAT_GLASS;
                    hm.tex[0] = read_texture(s, scene_stream, sub_images);
                    hm.tex[1] = read_texture(s, scene_stream, sub_images);
                    break;
                case 'M': hm.kind = MAT_NONE; break;
                case 'C':
                    hm.kind = MAT_METAL;
                    hm.tex[0] = read_texture(s, scene_stream, sub_images);
                    hm.tex[1] = read_texture(s, scene_stream, sub_images);
                    if (hm.tex[1].kind != TEX_CONSTANT)
                        throw ParseError{LTS_ERR_PARSE, "conductor eta must be a constant ('c') record"};
                    break;
                default: throw ParseError{LTS_ERR_PARSE, std::string("unknown material type '") + ty + "'"};
            }
            hm.extra = tokf(s, "material extra parameter");
            for (const HostTexture& t : hm.tex)  // setMatTexture indexes the mipmaps unchecked
                if (t.kind == TEX_IMAGE && !(t.v[0] >= 0.0f && (int)t.v[0] < images))
                    throw ParseError{LTS_ERR_PARSE, "image texture index out of range"};
            if (hm.kind == MAT_MATTE && hm.extra != 0) {  // OrenNayar ctor, Microfacet.cuh:18-25
                const float sigma = (float)((double)hm.extra * (kPi / 180));  // toRadians, GeneralHelper.cuh
                const float sigma2 = sigma * sigma;
                hm.on_a = 1.0f - (sigma2 / (2.0f * (sigma2 + 0.33f)));
                hm.on_b = 0.45f * sigma2 / (sigma2 + 0.09f);
            }
            sc->materials.push_back(hm);
        }
        // Lights (SceneLoader.cuh:173-193).
        const int area_meshes = toki(ss, "area light mesh count");
        std::vector<float> les;
        for (int i = 0; i < 3 * area_meshes; ++i) les.push_back(tokf(ss, "area light Le"));
        const bool has_inf = toki(ss, "infinite light flag") > 0;
        float inf_le[3] = {0, 0, 0};
        if (has_inf)
            for (int i = 0; i < 3; ++i) inf_le[i] = tokf(ss, "infinite light Le");
        // Grammar extension (no counterpart in the reference, whose PointLight, Light.cuh:53-86,
        // no file can create): after the infinite-light record, the keyword `pointLights`, a
        // count, and per light `px py pz  Ir Ig Ib` (world-space position, intensity).  The
        // reference stops reading after the infinite-light record, so it loads such a file
        // without its point lights; anything else there (platforms/plane.scene keeps a comment
        // and a material record) is ignored here too.
        // A second extension record, `instances K` and per instance `meshIndex tx ty tz s`: mesh
        // entry meshIndex (in the global mesh order, subject meshes first) is an instance of its
        // mesh file, placed at p * s + t (s > 0).  Entries that name the same file share one
        // prototype; the renderer's 8-wide BVH then holds one bottom-level tree per prototype and
        // a top level over the instances, instead of every copy's triangles.  Emissive meshes
        // cannot be instanced.
        std::vector<float> points;
        std::vector<HostInstance> inst;
        {
            std::string t;
            bool more = ss.next(&t);
            while (more && (t == "pointLights" || t == "instances")) {
                if (t == "pointLights") {
                    const int np = toki(ss, "point light count");
                    if (np < 0) throw ParseError{LTS_ERR_PARSE, "negative point light count"};
                    for (int i = 0; i < 6 * np; ++i) points.push_back(tokf(ss, "point light position / intensity"));
                } else {
                    const int ni = toki(ss, "instance count");
                    if (ni < 0) throw ParseError{LTS_ERR_PARSE, "negative instance count"};
                    for (int i = 0; i < ni; ++i) {
                        HostInstance h;
                        h.mesh = toki(ss, "instance mesh index");
                        for (int c = 0; c < 3; ++c) h.t[c] = tokf(ss, "instance translation");
                        h.s = tokf(ss, "instance scale");
                        if (!(h.s > 0.0f)) throw ParseError{LTS_ERR_PARSE, "instance scale must be > 0"};
                        inst.push_back(h);
                    }
                }
                more = ss.next(&t);
            }
        }
        if (area_meshes < 0 || area_meshes > meshes)
            throw ParseError{LTS_ERR_PARSE, "area light mesh count exceeds mesh count"};
        if (mats < meshes)
            throw ParseError{LTS_ERR_PARSE, "fewer materials than meshes (material index == mesh index)"};
        // instance of mesh entry m (-1: none); prototypes by mesh file
        std::vector<int32_t> inst_of(meshes, -1);
        sc->instances.clear();
        sc->proto_soup.clear();
        {
            std::vector<std::string> proto_files;
            if (inst.size() > (size_t)kMaxSceneInstances)
                throw ParseError{LTS_ERR_PARSE, "more than " + std::to_string(kMaxSceneInstances) + " instances"};
            // the renderer's two-level BVH applies p * s + t alone, so a subject mesh is instanced
            // only under the identity subject transform (rotation by 0, scale 1, no translation)
            const bool xf_identity = subject_xf.t.x == 0.0f && subject_xf.t.y == 0.0f && subject_xf.t.z == 0.0f &&
                                     subject_xf.r.w == 1.0f && subject_xf.r.x == 0.0f && subject_xf.r.y == 0.0f &&
                                     subject_xf.r.z == 0.0f && subject_xf.s == 1.0f;
            for (size_t k = 0; k < inst.size(); ++k) {
                HostInstance h = inst[k];
                if (h.mesh < 0 || h.mesh >= meshes) throw ParseError{LTS_ERR_PARSE, "instance mesh index out of range"};
                if (inst_of[h.mesh] >= 0) throw ParseError{LTS_ERR_PARSE, "mesh entry instanced twice"};
                if (h.mesh >= meshes - area_meshes) throw ParseError{LTS_ERR_PARSE, "an emissive mesh cannot be instanced"};
                if (h.mesh < sub_meshes && !xf_identity)
                    throw ParseError{LTS_ERR_PARSE, "an instanced subject mesh needs the identity subject transform"};
                h.proto = -1;
                for (size_t q = 0; q < proto_files.size(); ++q)
                    if (proto_files[q] == files[h.mesh]) h.proto = (int32_t)q;
                if (h.proto < 0) {
                    h.proto = (int32_t)proto_files.size();
                    proto_files.push_back(files[h.mesh]);
                }
                inst_of[h.mesh] = (int32_t)sc->instances.size();
                sc->instances.push_back(h);
            }
            sc->proto_soup.resize(proto_files.size());
        }

        // Mesh loading + transforms (SceneLoader.cuh:264-282, shapes/Triangle.cu:20-43).
        // Every mesh is read (and checked) first, so each table is sized once; each mesh then
        // fills its own ranges of them in parallel.
        std::vector<MeshData> mds(meshes);
        size_t np_all = 0, nn_all = 0, nuv_all = 0, nt_all = 0;
        for (int m = 0; m < meshes; ++m) {
            mds[m] = read_mesh(files[m]);
            check_indices(mds[m], files[m]);
            np_all += (size_t)mds[m].np;
            nn_all += (size_t)mds[m].nn;
            nuv_all += (size_t)mds[m].nuv;
            nt_all += (size_t)mds[m].ntri;
        }
        if (nt_all > (size_t)INT32_MAX / 3 || np_all > (size_t)INT32_MAX / 3)
            throw ParseError{LTS_ERR_PARSE, "scene too large"};
        sc->p.resize(3 * np_all);
        sc->n.resize(3 * nn_all);
        sc->uv.resize(2 * nuv_all);
        sc->tri_p.resize(3 * nt_all);
        sc->tri_n.resize(3 * nt_all);
        sc->tri_uv.resize(3 * nt_all);
        sc->tri_mesh.resize(nt_all);
        sc->mesh_first_tri.clear();
        sc->mesh_tri_count.clear();
        const Xform ident;  // Transform(1)
        size_t pbase = 0, nbase = 0, uvbase = 0, tbase = 0;
        for (int m = 0; m < meshes; ++m) {
            const MeshData& md = mds[m];
            const Xform& X = m >= sub_meshes ? ident : subject_xf;
            const float *mp = md.P(), *mn = md.N(), *muv = md.UV();
            const int32_t* mi = md.I();
            const HostInstance* hi = inst_of[m] >= 0 ? &sc->instances[inst_of[m]] : nullptr;
            parallel_ranges((size_t)md.np, [&](size_t b, size_t e) {
                for (size_t i = b; i < e; ++i) {
                    V3 q{mp[3 * i], mp[3 * i + 1], mp[3 * i + 2]};
                    if (hi) q = V3{q.x * hi->s + hi->t[0], q.y * hi->s + hi->t[1], q.z * hi->s + hi->t[2]};
                    const V3 w = X.point(q);
                    float* o = &sc->p[3 * (pbase + i)];
                    o[0] = w.x; o[1] = w.y; o[2] = w.z;
                }
            });
            if (hi && sc->proto_soup[hi->proto].empty()) {  // the prototype's object-space triangles
                std::vector<float>& soup = sc->proto_soup[hi->proto];
                soup.resize(9 * (size_t)md.ntri);
                for (int32_t t = 0; t < md.ntri; ++t)
                    for (int c = 0; c < 3; ++c)
                        for (int k = 0; k < 3; ++k) soup[9 * (size_t)t + 3 * c + k] = mp[3 * (size_t)mi[9 * t + 3 * c] + k];
            }
            parallel_ranges((size_t)md.nn, [&](size_t b, size_t e) {
                for (size_t i = b; i < e; ++i) {
                    const V3 w = X.normal({mn[3 * i], mn[3 * i + 1], mn[3 * i + 2]});
                    float* o = &sc->n[3 * (nbase + i)];
                    o[0] = w.x; o[1] = w.y; o[2] = w.z;
                }
            });
            if (md.nuv > 0) std::memcpy(&sc->uv[2 * uvbase], muv, 8 * (size_t)md.nuv);
            sc->mesh_first_tri.push_back((int32_t)tbase);
            sc->mesh_tri_count.push_back(md.ntri);
            const int32_t pb = (int32_t)pbase, nb = (int32_t)nbase, ub = (int32_t)uvbase;
            const bool has_uv = md.nuv > 0, has_n = md.nn > 0;
            parallel_ranges((size_t)md.ntri, [&](size_t b, size_t e) {
                for (size_t t = b; t < e; ++t) {
                    for (int c = 0; c < 3; ++c) {
                        const size_t o = 3 * (tbase + t) + c;
                        sc->tri_p[o] = pb + mi[9 * t + 3 * c];
                        sc->tri_uv[o] = has_uv ? ub + mi[9 * t + 3 * c + 1] : -1;
                        sc->tri_n[o] = has_n ? nb + mi[9 * t + 3 * c + 2] : -1;
                    }
                    sc->tri_mesh[tbase + t] = m;
                }
            });
            pbase += (size_t)md.np;
            nbase += (size_t)md.nn;
            uvbase += (size_t)md.nuv;
            tbase += (size_t)md.ntri;
        }
        sc->subject_meshes = sub_meshes;
        sc->area_light_meshes = area_meshes;
        sc->has_infinite = has_inf;
        const int32_t ntri = sc->triangles();
        if (ntri < 1) throw ParseError{LTS_ERR_PARSE, "scene has no triangles"};

        // Lights (SceneLoader_kernels.cu:52-111).  With one emissive mesh this is the
        // reference's array exactly (slot = triangle index within the mesh); several emissive
        // meshes race for the same slots in the reference, and are concatenated here.
        sc->lights.clear();
        sc->prim_light.assign(ntri, -1);
        for (int m = meshes - area_meshes; m < meshes; ++m) {
            const int le = meshes - m - 1;  // Le listed in reverse mesh order
            for (int32_t k = 0; k < sc->mesh_tri_count[m]; ++k) {
                HostLight L;
                L.kind = LIGHT_AREA;
                L.prim = sc->mesh_first_tri[m] + k;
                for (int c = 0; c < 3; ++c) L.L[c] = les[3 * le + c];
                const float* P = sc->p.data();
                const int32_t* ti = &sc->tri_p[3 * (size_t)L.prim];
                V3 p0{P[3 * ti[0]], P[3 * ti[0] + 1], P[3 * ti[0] + 2]};
                V3 p1{P[3 * ti[1]], P[3 * ti[1] + 1], P[3 * ti[1] + 2]};
                V3 p2{P[3 * ti[2]], P[3 * ti[2] + 1], P[3 * ti[2] + 2]};
                V3 c = cross_d(sub(p1, p0), sub(p2, p0));
                L.area = 0.5f * sqrtf(len2(c));  // Triangle.cuh:57-62
                sc->prim_light[L.prim] = (int32_t)sc->lights.size();
                sc->lights.push_back(L);
            }
        }
        // point lights (the extension above) come after the area lights and before the
        // infinite light: PointLight(LTW, I) at LTW(0, 0, 0) (Light.cuh:60-61)
        for (size_t k = 0; k + 6 <= points.size(); k += 6) {
            HostLight L;
            L.kind = LIGHT_POINT;
            for (int c = 0; c < 3; ++c) {
                L.p[c] = points[k + c];
                L.L[c] = points[k + 3 + c];
            }
            sc->lights.push_back(L);
        }
        if (has_inf) {
            HostLight L;
            L.kind = LIGHT_INFINITE;
            for (int c = 0; c < 3; ++c) L.L[c] = inf_le[c];
            // preprocess(info->bounds[0]) (SceneLoader_kernels.cu:102): triangle 0's AABB.
            const float* P = sc->p.data();
            float mn[3], mx[3];
            for (int k = 0; k < 3; ++k) {
                const float a = P[3 * sc->tri_p[0] + k], b = P[3 * sc->tri_p[1] + k], c = P[3 * sc->tri_p[2] + k];
                mn[k] = fminf(fminf(a, b), c);
                mx[k] = fmaxf(fmaxf(a, b), c);
            }
            for (int k = 0; k < 3; ++k) L.p[k] = mn[k] * 0.5f + mx[k] * 0.5f;  // Light.cuh:136-139
            V3 d{mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
            L.radius = sqrtf(len2(d)) / 2.0f;
            sc->lights.push_back(L);
        }
        // Light power distribution (IntegratorHelper.cuh:147-162, Sampling.cuh:123-144).
        const int nl = (int)sc->lights.size();
        sc->light_func.assign(nl, 0.f);
        for (int l = 0; l < nl; ++l) {
            const HostLight& L = sc->lights[l];
            float s[3];
            if (L.kind == LIGHT_AREA) {
                for (int c = 0; c < 3; ++c) s[c] = (L.L[c] * L.area) * (float)kPi;  // Light.cuh:104-106
            } else if (L.kind == LIGHT_INFINITE) {
                const float v = (float)(kPi * (double)L.radius);  // Light.cuh:141-143
                for (int c = 0; c < 3; ++c) s[c] = L.L[c] * v;
            } else {
                const float v = (float)(4 * kPi);  // Light.cuh:83-85
                for (int c = 0; c < 3; ++c) s[c] = L.L[c] * v;
            }
            sc->light_func[l] = 0.212671f * s[0] + 0.715160f * s[1] + 0.072169f * s[2];  // Spectrum.cuh:217-220
        }
        sc->light_cdf.assign(nl + 1, 0.f);
        for (int i = 1; i < nl + 1; ++i) sc->light_cdf[i] = sc->light_cdf[i - 1] + sc->light_func[i - 1] / nl;
        const float func_int = sc->light_cdf[nl];
        sc->light_func_int = func_int;
        if (func_int == 0) {
            for (int i = 1; i < nl + 1; ++i) sc->light_cdf[i] = (float)i / (float)nl;
        } else {
            for (int i = 1; i < nl + 1; ++i) sc->light_cdf[i] /= func_int;
        }

        // Camera (rendering/Camera.cu:9-43), aperture 0 (LightTransportSimulation.cu:70).
        sc->width = width;
        sc->height = height;
        build_camera(cf, width, height, sc->cam);
        // Gaussian filter table (Filter.cuh:32-50,82-99): radius (1,1), alpha 1.
        {
            const float alpha = 1.0f, rx = 1.0f, ry = 1.0f;
            const float expx = expf(-alpha * rx * rx), expy = expf(-alpha * ry * ry);
            for (int y = 0; y < 16; ++y)
                for (int x = 0; x < 16; ++x) {
                    const float px = (x + 0.5f) * rx / 16, py = (y + 0.5f) * ry / 16;
                    const float gx = fmaxf(0, expf(-alpha * px * px) - expx);
                    const float gy = fmaxf(0, expf(-alpha * py * py) - expy);
                    sc->filter[y * 16 + x] = gx * gy;
                }
        }
    } catch (const ParseError& e) {
        *code = e.code;
        return e.msg;
    } catch (const std::bad_alloc&) {
        *code = LTS_ERR_OOM;
        return "out of host memory";
    } catch (const std::exception& e) {  // e.g. std::system_error when a loader thread cannot start
        *code = LTS_ERR_IO;
        return std::string("load failed: ") + e.what();
    }
    return "";
}

}  // namespace lts
