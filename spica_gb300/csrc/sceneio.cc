// sceneio.cc -- the reference's scene-file front-end, restated for the GB300 path: its
// XML scene format (spica/sceneparser.cc:72-335), binary PLY meshes (core/meshio.cc:76-
// 169), OBJ meshes (core/meshio.cc:170-250 over the tinyobjloader library) and Radiance
// .hdr environment maps (core/image.cc:252-385), read into the flat arrays that
// spgpu_upload_scene and spgpu_render take.  Host code only.
//
// The XML semantics follow SceneParser:
//   * elements are visited depth first; an element's children are stored before the
//     element itself (parseChildren), into one typed parameter store
//     (core/renderparams.h) that outlives the element, so values persist until a later
//     element consumes ("removes") them;
//   * integer / float / string / rgb / spectrum / transform store typed values under
//     their name; a string named "filename" is resolved against the scene file's folder;
//   * every other element creates a plugin object from the store (its parameters read
//     as the reference's plugin constructors read them, with or without removal) and
//     stores it under its name, else under its id and under its element name;
//   * <ref id> makes the object with that id the pending "bsdf";
//   * a <shape> consumes the pending bsdf and toWorld; with a pending <emitter
//     type="area"> every triangle becomes an area light of the stored "radiance";
//   * <transform> children compose as trans = sub * trans, rotate's angle is used as
//     radians (core/transform.cc:136), lookAt is Transform::lookAt.
// Only what the GPU path renders is accepted: perspective sensors (no depth of field),
// hdr / ldr films, the independent sampler, the path and direct-lighting integrators
// (and the gpupath / gpudirect drop-ins), BSDFs diffuse, roughconductor, dielectric,
// roughdielectric and plastic with constant parameters, PLY and OBJ meshes,
// area lights and an untransformed .hdr environment map.  Anything else is refused
// with the element and the reason.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spica_gpu.h"

namespace spgpu {
void setError(const std::string &msg);
}

namespace {

using spgpu::setError;

// ---------------------------------------------------------------- XML subset
struct XmlElem {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlElem> kids;
    int line = 0;
    const char *attr(const char *n) const {
        for (const auto &a : attrs)
            if (a.first == n) return a.second.c_str();
        return nullptr;
    }
};

class XmlReader {
public:
    explicit XmlReader(const std::string &text) : s_(text) {}

    bool document(XmlElem *root) {
        if (s_.compare(0, 3, "\xEF\xBB\xBF") == 0) i_ = 3;
        for (;;) {
            skipSpace();
            if (i_ >= s_.size()) return fail("no root element");
            if (starts("<?")) {
                if (!skipPast("?>")) return fail("unterminated declaration");
            } else if (starts("<!--")) {
                if (!skipPast("-->")) return fail("unterminated comment");
            } else if (starts("<!")) {
                if (!skipPast(">")) return fail("unterminated document type");
            } else if (s_[i_] == '<') {
                return element(root);
            } else {
                return fail("text before the root element");
            }
        }
    }
    const std::string &error() const { return err_; }

private:
    bool fail(const std::string &m) {
        if (err_.empty()) err_ = "line " + std::to_string(lineAt(i_)) + ": " + m;
        return false;
    }
    int lineAt(size_t p) const {
        int n = 1;
        for (size_t k = 0; k < p && k < s_.size(); k++) n += s_[k] == '\n';
        return n;
    }
    bool starts(const char *t) const { return s_.compare(i_, std::strlen(t), t) == 0; }
    bool skipPast(const char *t) {
        const size_t p = s_.find(t, i_);
        if (p == std::string::npos) return false;
        i_ = p + std::strlen(t);
        return true;
    }
    void skipSpace() {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) i_++;
    }
    static bool nameChar(char c) {
        return std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' || c == ':' || c == '.';
    }
    std::string name() {
        const size_t b = i_;
        while (i_ < s_.size() && nameChar(s_[i_])) i_++;
        return s_.substr(b, i_ - b);
    }
    bool decode(const std::string &raw, std::string *out) {
        out->clear();
        for (size_t k = 0; k < raw.size(); k++) {
            if (raw[k] != '&') {
                *out += raw[k];
                continue;
            }
            const size_t e = raw.find(';', k);
            if (e == std::string::npos) return fail("unterminated character reference");
            const std::string ent = raw.substr(k + 1, e - k - 1);
            if (ent == "lt") *out += '<';
            else if (ent == "gt") *out += '>';
            else if (ent == "amp") *out += '&';
            else if (ent == "quot") *out += '"';
            else if (ent == "apos") *out += '\'';
            else if (!ent.empty() && ent[0] == '#') {
                const long v = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? std::strtol(ent.c_str() + 2, nullptr, 16)
                                                                                   : std::strtol(ent.c_str() + 1, nullptr, 10);
                if (v <= 0 || v > 127) return fail("character reference outside ASCII");
                *out += static_cast<char>(v);
            } else {
                return fail("unknown entity &" + ent + ";");
            }
            k = e;
        }
        return true;
    }
    bool element(XmlElem *el) {
        el->line = lineAt(i_);
        i_++;   // '<'
        el->name = name();
        if (el->name.empty()) return fail("element without a name");
        for (;;) {
            skipSpace();
            if (i_ >= s_.size()) return fail("unterminated element <" + el->name + ">");
            if (starts("/>")) {
                i_ += 2;
                return true;
            }
            if (s_[i_] == '>') {
                i_++;
                break;
            }
            const std::string an = name();
            if (an.empty()) return fail("bad attribute in <" + el->name + ">");
            skipSpace();
            if (i_ >= s_.size() || s_[i_] != '=') return fail("attribute " + an + " without a value");
            i_++;
            skipSpace();
            if (i_ >= s_.size() || (s_[i_] != '"' && s_[i_] != '\'')) return fail("unquoted attribute " + an);
            const char q = s_[i_++];
            const size_t e = s_.find(q, i_);
            if (e == std::string::npos) return fail("unterminated attribute " + an);
            std::string v;
            if (!decode(s_.substr(i_, e - i_), &v)) return false;
            i_ = e + 1;
            el->attrs.emplace_back(an, v);
        }
        // content: child elements, comments, text (ignored)
        for (;;) {
            if (i_ >= s_.size()) return fail("unterminated element <" + el->name + ">");
            if (starts("</")) {
                i_ += 2;
                const std::string close = name();
                skipSpace();
                if (close != el->name || i_ >= s_.size() || s_[i_] != '>')
                    return fail("</" + close + "> does not close <" + el->name + ">");
                i_++;
                return true;
            }
            if (starts("<!--")) {
                if (!skipPast("-->")) return fail("unterminated comment");
            } else if (starts("<![CDATA[")) {
                if (!skipPast("]]>")) return fail("unterminated CDATA section");
            } else if (starts("<?")) {
                if (!skipPast("?>")) return fail("unterminated processing instruction");
            } else if (s_[i_] == '<') {
                el->kids.emplace_back();
                if (!element(&el->kids.back())) return false;
            } else {
                i_++;
            }
        }
    }

    const std::string &s_;
    size_t i_ = 0;
    std::string err_;
};

// ---------------------------------------------------------------- transforms
struct Mat4 {
    double m[4][4];
    static Mat4 identity() {
        Mat4 r{};
        for (int i = 0; i < 4; i++) r.m[i][i] = 1.0;
        return r;
    }
    Mat4 operator*(const Mat4 &b) const {
        Mat4 r{};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                r.m[i][j] = m[i][0] * b.m[0][j] + m[i][1] * b.m[1][j] + m[i][2] * b.m[2][j] + m[i][3] * b.m[3][j];
        return r;
    }
    bool isIdentity() const {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                if (m[i][j] != (i == j ? 1.0 : 0.0)) return false;
        return true;
    }
    // Transform::apply(Point3d) (core/transform.cc:60-76), with its projective division
    // by w + 1e-12 when w is not 1
    void point(const double p[3], double out[3]) const {
        double r[4];
        for (int i = 0; i < 4; i++) r[i] = m[i][0] * p[0] + m[i][1] * p[1] + m[i][2] * p[2] + m[i][3];
        for (int i = 0; i < 3; i++) out[i] = r[3] != 1.0 ? r[i] / (r[3] + 1.0e-12) : r[i];
    }
    void vector(const double v[3], double out[3]) const {
        for (int i = 0; i < 3; i++) out[i] = m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2];
    }
};

void normalize3(double v[3]) {
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; i++) v[i] /= n;
}
void cross3(const double a[3], const double b[3], double r[3]) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// Transform::translate / scale / rotate / lookAt (core/transform.cc:110-204)
Mat4 translate(double x, double y, double z) {
    Mat4 r = Mat4::identity();
    r.m[0][3] = x;
    r.m[1][3] = y;
    r.m[2][3] = z;
    return r;
}
Mat4 scale(double x, double y, double z) {
    Mat4 r = Mat4::identity();
    r.m[0][0] = x;
    r.m[1][1] = y;
    r.m[2][2] = z;
    return r;
}
Mat4 rotate(double theta, const double axis[3]) {
    double a[3] = {axis[0], axis[1], axis[2]};
    normalize3(a);
    const double s = std::sin(theta), c = std::cos(theta);
    Mat4 r{};
    r.m[0][0] = a[0] * a[0] + (1.0 - a[0] * a[0]) * c;
    r.m[0][1] = a[0] * a[1] * (1.0 - c) - a[2] * s;
    r.m[0][2] = a[0] * a[2] * (1.0 - c) + a[1] * s;
    r.m[1][0] = a[0] * a[1] * (1.0 - c) + a[2] * s;
    r.m[1][1] = a[1] * a[1] + (1.0 - a[1] * a[1]) * c;
    r.m[1][2] = a[1] * a[2] * (1.0 - c) - a[0] * s;
    r.m[2][0] = a[0] * a[2] * (1.0 - c) - a[1] * s;
    r.m[2][1] = a[1] * a[2] * (1.0 - c) + a[0] * s;
    r.m[2][2] = a[2] * a[2] + (1.0 - a[2] * a[2]) * c;
    r.m[3][3] = 1.0;
    return r;
}
bool lookAt(const double eye[3], const double look[3], const double up[3], Mat4 *out) {
    double dir[3] = {look[0] - eye[0], look[1] - eye[1], look[2] - eye[2]};
    normalize3(dir);
    double un[3] = {up[0], up[1], up[2]};
    normalize3(un);
    double left[3];
    cross3(un, dir, left);
    if (std::sqrt(left[0] * left[0] + left[1] * left[1] + left[2] * left[2]) == 0.0) return false;
    normalize3(left);
    double nup[3];
    cross3(dir, left, nup);
    Mat4 r{};
    for (int i = 0; i < 3; i++) {
        r.m[i][0] = left[i];
        r.m[i][1] = nup[i];
        r.m[i][2] = dir[i];
        r.m[i][3] = eye[i];
    }
    r.m[3][3] = 1.0;
    *out = r;
    return true;
}

// ---------------------------------------------------------------- parameter store
struct Object {
    std::string element, type;
    float material[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // bsdf
    int width = 0, height = 0;                       // film
    Mat4 toWorld = Mat4::identity();                 // sensor, envmap
    double fov = 0.0;                                // sensor, degrees
    std::shared_ptr<Object> film;                    // sensor
    std::vector<float> env;                          // envmap, RGB
    int envW = 0, envH = 0;
};
using ObjectPtr = std::shared_ptr<Object>;

struct Spectrum3 {
    double v[3];
};

template <class T>
struct Table {
    std::map<std::string, T> map;
    bool get(const std::string &n, T *out, bool remove) {
        auto it = map.find(n);
        if (it == map.end()) return false;
        *out = it->second;
        if (remove) map.erase(it);
        return true;
    }
};

struct Store {
    Table<int> ints;
    Table<double> doubles;
    Table<std::string> strings;
    Table<Spectrum3> spectra;
    Table<Mat4> transforms;
    Table<ObjectPtr> objects;
    Table<bool> bools;
    // RenderParams::getTexture (core/renderparams.cc:374-462): an object, else a
    // spectrum, else a double, as a constant; objects (image textures) are refused
    int texture(const std::string &n, double out[3], bool remove, std::string *why) {
        ObjectPtr o;
        if (objects.get(n, &o, remove)) {
            *why = "texture objects are not supported (" + n + ")";
            return -1;
        }
        Spectrum3 s;
        if (spectra.get(n, &s, remove)) {
            for (int i = 0; i < 3; i++) out[i] = s.v[i];
            return 1;
        }
        double d;
        if (doubles.get(n, &d, remove)) {
            out[0] = out[1] = out[2] = d;
            return 1;
        }
        return 0;
    }
};

// gray value of the reference's RGB spectrum (core/spectrum.cc:677)
double grayOf(const double v[3]) { return 0.2126 * v[0] + 0.7152 * v[1] + 0.0722 * v[2]; }

// ---------------------------------------------------------------- meshes and images
// meshio::loadPLY (core/meshio.cc:76-169): "ply", binary little endian, the header's
// vertex and face counts; vertices are three floats (other vertex properties are not
// read), faces a one-byte count and three int32 indices (only the first triangle of a
// polygon; its extra indices are skipped)
bool loadPly(const std::string &path, const Mat4 &toWorld, std::vector<float> *tris, std::string *why) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        *why = "cannot open " + path;
        return false;
    }
    std::string line;
    std::getline(f, line);
    if (line != "ply") {
        *why = path + ": not a PLY file";
        return false;
    }
    long nv = 0, nf = 0;
    for (;;) {
        if (!std::getline(f, line)) {
            *why = path + ": no end_header";
            return false;
        }
        std::stringstream ss(line);
        std::string key, name, val;
        ss >> key;
        if (key == "format") {
            ss >> name >> val;
            if (name != "binary_little_endian") {
                *why = path + ": PLY must be binary little endian";
                return false;
            }
        } else if (key == "element") {
            ss >> name;
            if (name == "vertex") ss >> nv;
            else if (name == "face") ss >> nf;
            else {
                *why = path + ": unknown PLY element " + name;
                return false;
            }
        } else if (key == "end_header") {
            break;
        }
    }
    if (nv <= 0 || nf <= 0) {
        *why = path + ": vertex and face counts must be positive";
        return false;
    }
    // the body holds 12 bytes per vertex and at least 13 per face: refuse counts that the
    // file cannot hold before allocating for them
    const std::streamoff body = f.tellg();
    f.seekg(0, std::ios::end);
    const std::streamoff avail = f.tellg() - body;
    f.seekg(body);
    if (body < 0 || nv > avail / 12 || nf > (avail - 12 * nv) / 13) {
        *why = path + ": truncated vertex data or face data (the header's counts exceed the file)";
        return false;
    }
    std::vector<double> v(3 * nv);
    for (long i = 0; i < nv; i++) {
        unsigned char b[12];
        if (!f.read(reinterpret_cast<char *>(b), 12)) {
            *why = path + ": truncated vertex data";
            return false;
        }
        for (int k = 0; k < 3; k++) {
            const uint32_t u = static_cast<uint32_t>(b[4 * k]) | static_cast<uint32_t>(b[4 * k + 1]) << 8 |
                               static_cast<uint32_t>(b[4 * k + 2]) << 16 | static_cast<uint32_t>(b[4 * k + 3]) << 24;
            float x;
            std::memcpy(&x, &u, 4);
            v[3 * i + k] = x;
        }
    }
    for (long i = 0; i < nf; i++) {
        unsigned char cnt;
        unsigned char b[12];
        if (!f.read(reinterpret_cast<char *>(&cnt), 1) || !f.read(reinterpret_cast<char *>(b), 12)) {
            *why = path + ": truncated face data";
            return false;
        }
        int32_t idx[3];
        for (int k = 0; k < 3; k++) {
            const uint32_t u = static_cast<uint32_t>(b[4 * k]) | static_cast<uint32_t>(b[4 * k + 1]) << 8 |
                               static_cast<uint32_t>(b[4 * k + 2]) << 16 | static_cast<uint32_t>(b[4 * k + 3]) << 24;
            std::memcpy(&idx[k], &u, 4);
            if (idx[k] < 0 || idx[k] >= nv) {
                *why = path + ": face index out of range";
                return false;
            }
        }
        for (int k = 0; k < 3; k++) {
            double p[3];
            toWorld.point(&v[3 * idx[k]], p);
            for (int c = 0; c < 3; c++) tris->push_back(static_cast<float>(p[c]));
        }
        if (cnt > 3) f.seekg(4 * (cnt - 3), std::ios::cur);
    }
    return true;
}

// OBJ through the published behaviour of tinyobjloader, which the reference calls
// (core/meshio.cc:170-250): "v x y z" positions; "f" faces of 1-based (or negative,
// relative) position indices, optionally with /texcoord/normal parts, triangulated as a
// fan around their first vertex; other statements ignored
bool loadObj(const std::string &path, const Mat4 &toWorld, std::vector<float> *tris, std::string *why) {
    std::ifstream f(path);
    if (!f) {
        *why = "cannot open " + path;
        return false;
    }
    std::vector<double> v;
    std::string line;
    int ln = 0;
    while (std::getline(f, line)) {
        ln++;
        std::stringstream ss(line);
        std::string key;
        ss >> key;
        if (key == "v") {
            double x, y, z;
            if (!(ss >> x >> y >> z)) {
                *why = path + ":" + std::to_string(ln) + ": bad vertex";
                return false;
            }
            v.push_back(x);
            v.push_back(y);
            v.push_back(z);
        } else if (key == "f") {
            std::vector<long> ids;
            std::string tok;
            while (ss >> tok) {
                const long k = std::strtol(tok.c_str(), nullptr, 10);
                const long nvert = static_cast<long>(v.size() / 3);
                const long idx = k > 0 ? k - 1 : nvert + k;
                if (k == 0 || idx < 0 || idx >= nvert) {
                    *why = path + ":" + std::to_string(ln) + ": face index out of range";
                    return false;
                }
                ids.push_back(idx);
            }
            for (size_t t = 2; t < ids.size(); t++) {
                const long tri[3] = {ids[0], ids[t - 1], ids[t]};
                for (int k = 0; k < 3; k++) {
                    double p[3];
                    toWorld.point(&v[3 * tri[k]], p);
                    for (int c = 0; c < 3; c++) tris->push_back(static_cast<float>(p[c]));
                }
            }
        }
    }
    return true;
}

// Image::loadHdr (core/image.cc:252-385): "#?RADIANCE", a "-Y H +X W" size line, then
// run-length-encoded scanlines (2, 2, width, then each channel as literal runs of up
// to 128 bytes and repeat runs of count-128); pixel = mantissa * 2^(e - 128) / 256
bool loadHdr(const std::string &path, std::vector<float> *rgb, int *W, int *H, std::string *why) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        *why = "cannot open " + path;
        return false;
    }
    std::string line;
    bool valid = false;
    for (;;) {
        if (!std::getline(f, line)) {
            *why = path + ": truncated header";
            return false;
        }
        if (!line.empty() && line[0] == '#' && line == "#?RADIANCE") valid = true;
        if (line.empty()) break;
    }
    if (!valid) {
        *why = path + ": not a Radiance HDR file";
        return false;
    }
    std::getline(f, line);
    char by[17] = {0}, bx[17] = {0};
    int w = 0, h = 0;
    if (std::sscanf(line.c_str(), "%16s %d %16s %d", by, &h, bx, &w) != 4 || std::strcmp(by, "-Y") != 0 ||
        std::strcmp(bx, "+X") != 0 || w <= 0 || h <= 0) {
        *why = path + ": unsupported HDR size line";
        return false;
    }
    if (w > 0x7FFF || static_cast<int64_t>(w) * h > (int64_t(1) << 28)) {   // RLE widths are 15-bit
        *why = path + ": image too large (width < 32768, at most 2^28 pixels)";
        return false;
    }
    std::vector<unsigned char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<unsigned char> px(static_cast<size_t>(w) * h * 4, 0);
    size_t i = 0;
    for (int y = 0; y < h && i + 4 <= bytes.size(); y++) {
        if (bytes[i] != 2 || bytes[i + 1] != 2) break;
        const int sw = bytes[i + 2] << 8 | bytes[i + 3];
        i += 4;
        if (sw != w) {
            *why = path + ": scanline width differs from the image width";
            return false;
        }
        for (int c = 0; c < 4; c++) {
            for (int x = 0; x < w;) {
                if (i >= bytes.size()) {
                    *why = path + ": truncated scanline";
                    return false;
                }
                const int info = bytes[i++];
                const int n = info <= 128 ? info : info - 128;
                if (n == 0 || x + n > w || (info <= 128 && i + n > bytes.size()) || (info > 128 && i >= bytes.size())) {
                    *why = path + ": bad run in scanline";
                    return false;
                }
                for (int k = 0; k < n; k++, x++)
                    px[(static_cast<size_t>(y) * w + x) * 4 + c] = info <= 128 ? bytes[i++] : bytes[i];
                if (info > 128) i++;
            }
        }
    }
    rgb->resize(static_cast<size_t>(w) * h * 3);
    for (size_t p = 0; p < static_cast<size_t>(w) * h; p++) {
        const double s = std::pow(2.0, px[4 * p + 3] - 128.0) / 256.0;
        for (int c = 0; c < 3; c++) (*rgb)[3 * p + c] = static_cast<float>(px[4 * p + c] * s);
    }
    *W = w;
    *H = h;
    return true;
}

// ---------------------------------------------------------------- the parser
struct Loaded {
    std::vector<float> verts, emit, materials;
    std::vector<int32_t> triMat;
    std::vector<float> env;
    int envW = 0, envH = 0;
    ObjectPtr camera;
    std::string integrator;
};

class Parser {
public:
    explicit Parser(const std::string &file) : file_(file) {
        const size_t s = file.find_last_of('/');
        dir_ = s == std::string::npos ? std::string(".") : file.substr(0, s);
        store_.ints.map["maxDepth"] = 16;   // SceneParser::SceneParser (spica/sceneparser.cc:62)
    }

    bool run(const XmlElem &root, Loaded *out) {
        out_ = out;
        if (root.name != "scene") return fail(root, "the root element must be <scene>");
        if (!children(root)) return false;
        if (!out_->camera) return fail(root, "no <sensor>");
        return true;
    }
    const std::string &error() const { return err_; }
    Store &store() { return store_; }

private:
    bool fail(const XmlElem &e, const std::string &m) {
        if (err_.empty()) err_ = file_ + ":" + std::to_string(e.line) + ": <" + e.name + ">: " + m;
        return false;
    }
    static bool number(const char *s, double *out) {
        if (!s) return false;
        char *end = nullptr;
        *out = std::strtod(s, &end);
        return end != s;
    }
    static bool triple(const char *s, double out[3]) {
        if (!s) return false;
        std::string t(s);
        for (auto &c : t)
            if (c == ',') c = ' ';
        std::stringstream ss(t);
        return static_cast<bool>(ss >> out[0] >> out[1] >> out[2]);
    }
    bool children(const XmlElem &parent) {
        for (const auto &e : parent.kids) {
            if (!e.kids.empty() && e.name != "transform" && !children(e)) return false;
            if (!store(e)) return false;
        }
        return true;
    }
    bool transform(const XmlElem &t, Mat4 *out) {
        Mat4 trans = Mat4::identity();
        for (const auto &e : t.kids) {
            Mat4 sub = Mat4::identity();
            double x, y, z, a;
            if (e.name == "matrix") {
                std::stringstream ss(e.attr("value") ? e.attr("value") : "");
                for (int i = 0; i < 16; i++)
                    if (!(ss >> sub.m[i / 4][i % 4])) return fail(e, "needs 16 values");
            } else if (e.name == "scale" || e.name == "translate" || e.name == "rotate") {
                if (!number(e.attr("x"), &x) || !number(e.attr("y"), &y) || !number(e.attr("z"), &z))
                    return fail(e, "needs x, y and z");
                if (e.name == "scale") {
                    sub = scale(x, y, z);
                } else if (e.name == "translate") {
                    sub = translate(x, y, z);
                } else {
                    if (!number(e.attr("angle"), &a)) return fail(e, "needs an angle");
                    const double axis[3] = {x, y, z};
                    sub = rotate(a, axis);
                }
            } else if (e.name == "lookAt") {
                double o[3], tg[3], up[3];
                if (!triple(e.attr("origin"), o) || !triple(e.attr("target"), tg) || !triple(e.attr("up"), up))
                    return fail(e, "needs origin, target and up");
                if (!lookAt(o, tg, up, &sub)) return fail(e, "up is parallel to the viewing direction");
            }
            trans = sub * trans;
        }
        *out = trans;
        return true;
    }
    std::string resolve(const std::string &p) const { return !p.empty() && p[0] == '/' ? p : dir_ + "/" + p; }

    bool store(const XmlElem &e) {
        const std::string &node = e.name;
        const std::string name = e.attr("name") ? e.attr("name") : "";
        double d;
        if (node == "boolean") {
            if (!name.empty()) store_.bools.map[name] = e.attr("value") && std::strcmp(e.attr("value"), "true") == 0;
        } else if (node == "integer") {
            if (!number(e.attr("value"), &d)) return fail(e, "needs a value");
            if (!name.empty()) store_.ints.map[name] = static_cast<int>(std::strtol(e.attr("value"), nullptr, 10));
        } else if (node == "float") {
            if (!number(e.attr("value"), &d)) return fail(e, "needs a value");
            if (!name.empty()) store_.doubles.map[name] = d;
        } else if (node == "string") {
            if (!e.attr("value")) return fail(e, "needs a value");
            std::string v = e.attr("value");
            if (name == "filename") v = resolve(v);
            if (!name.empty()) store_.strings.map[name] = v;
        } else if (node == "rgb") {
            Spectrum3 s;
            if (!triple(e.attr("value"), s.v)) return fail(e, "needs three values");
            if (!name.empty()) store_.spectra.map[name] = s;
        } else if (node == "spectrum") {
            return fail(e, "sampled spectra are not supported");
        } else if (node == "transform") {
            Mat4 t;
            if (!transform(e, &t)) return false;
            if (!name.empty()) store_.transforms.map[name] = t;
        } else if (node == "shape") {
            return shape(e);
        } else if (node == "ref") {
            const char *id = e.attr("id");
            ObjectPtr o;
            if (!id || !store_.objects.get(id, &o, false)) return fail(e, std::string("no object with id ") + (id ? id : ""));
            if (o->element == "bsdf") store_.objects.map["bsdf"] = o;
        } else if (node == "integrator") {
            const char *type = e.attr("type");
            if (!type || !*type) return fail(e, "no type");
            store_.strings.map["integrator"] = type;
            const std::string t = type;
            if (t == "path" || t == "gpupath") out_->integrator = "path";
            else if (t == "directlighting" || t == "gpudirect") out_->integrator = "direct";
            else return fail(e, "integrator type " + t + " has no GPU counterpart");
        } else {
            const char *type = e.attr("type");
            if (!type || !*type) return fail(e, "no type");
            if (node == "emitter" && std::strcmp(type, "area") == 0) {
                waitArea_ = true;
                return true;
            }
            ObjectPtr o = std::make_shared<Object>();
            o->element = node;
            o->type = type;
            if (!create(e, o.get())) return false;
            if (!name.empty()) {
                store_.objects.map[name] = o;
            } else {
                if (e.attr("id") && *e.attr("id")) store_.objects.map[e.attr("id")] = o;
                store_.objects.map[node] = o;
            }
            if (node == "sensor") {
                if (out_->camera) return fail(e, "a second sensor");
                out_->camera = o;
            } else if (node == "emitter") {
                if (!out_->env.empty()) return fail(e, "a second environment map");
                out_->env = o->env;
                out_->envW = o->envW;
                out_->envH = o->envH;
            }
        }
        return true;
    }

    // the plugins' constructors, reading the store as the reference's do
    bool create(const XmlElem &e, Object *o) {
        const std::string &t = o->type;
        std::string why;
        double a[3], b[3], c[3];
        float *M = o->material;
        auto tex = [&](const char *n, double *v, bool remove, const double *dflt) -> bool {
            const int r = store_.texture(n, v, remove, &why);
            if (r < 0) return fail(e, why);
            if (r == 0) {
                if (!dflt) return fail(e, std::string("needs ") + n);
                for (int i = 0; i < 3; i++) v[i] = dflt[i];
            }
            return true;
        };
        if (o->element == "bsdf") {
            double bump[3];
            if (store_.texture("bumpMap", bump, t == "diffuse" || t == "roughconductor", &why) != 0)
                return fail(e, "bump maps are not supported");
            const double alpha0[3] = {0.1, 0.1, 0.1};
            if (t == "diffuse") {   // bsdfs/diffuse.cc:19
                if (!tex("reflectance", a, true, nullptr)) return false;
                M[0] = SPGPU_MAT_LAMBERT;
                for (int i = 0; i < 3; i++) M[1 + i] = static_cast<float>(a[i]);
            } else if (t == "roughconductor") {   // bsdfs/roughconductor.cc:30-35
                std::string dist = "beckmann";
                if (!tex("eta", a, true, nullptr) || !tex("k", b, true, nullptr) || !tex("alpha", c, false, alpha0))
                    return false;
                store_.strings.get("distribution", &dist, true);
                if (dist != "ggx" && dist != "beckmann") return fail(e, "unknown distribution " + dist);
                M[0] = dist == "ggx" ? SPGPU_MAT_CONDUCTOR : SPGPU_MAT_CONDUCTOR_BECKMANN;
                M[1] = static_cast<float>(grayOf(c));
                for (int i = 0; i < 3; i++) {
                    M[2 + i] = static_cast<float>(a[i]);
                    M[5 + i] = static_cast<float>(b[i]);
                }
            } else if (t == "dielectric" || t == "roughdielectric") {   // bsdfs/dielectric.cc:24, roughdielectric.cc:32
                const double ior0[3] = {t == "dielectric" ? 1.333 : 1.3333, 0, 0};
                double ior[3];
                if (!tex("specularReflectance", a, false, nullptr) || !tex("specularTransmittance", b, false, nullptr))
                    return false;
                if (t == "roughdielectric" && !tex("alpha", c, false, alpha0)) return false;
                const double iorD[3] = {ior0[0], ior0[0], ior0[0]};
                if (!tex("intIOR", ior, false, iorD)) return false;
                for (int i = 0; i < 3; i++)
                    if (std::fmin(a[i], 1.0) != 1.0 || std::fmin(b[i], 1.0) != 1.0)
                        return fail(e, "only white specular reflectance and transmittance have a GPU counterpart");
                std::string dist = "beckmann";
                if (t == "roughdielectric") store_.strings.get("distribution", &dist, true);
                if (dist != "beckmann" && dist != "ggx") return fail(e, "unknown distribution " + dist);
                if (t == "dielectric" || grayOf(c) == 0.0) {
                    M[0] = SPGPU_MAT_DIELECTRIC;
                    M[1] = static_cast<float>(grayOf(ior));
                } else {
                    M[0] = SPGPU_MAT_ROUGH_DIELECTRIC;
                    M[1] = static_cast<float>(grayOf(c));
                    M[2] = static_cast<float>(grayOf(ior));
                    M[3] = dist == "ggx" ? 1.0f : 0.0f;
                }
            } else if (t == "plastic") {   // bsdfs/plastic.cc:105-108
                const double iorD[3] = {1.5, 1.5, 1.5};
                double ior[3];
                if (!tex("diffuseReflectance", a, false, nullptr) || !tex("specularReflectance", b, false, nullptr) ||
                    !tex("intIOR", ior, false, iorD))
                    return false;
                M[0] = SPGPU_MAT_PLASTIC;
                for (int i = 0; i < 3; i++) {
                    M[1 + i] = static_cast<float>(a[i]);
                    M[4 + i] = static_cast<float>(b[i]);
                }
                M[7] = static_cast<float>(grayOf(ior));
            } else {
                return fail(e, "bsdf type " + t + " has no GPU counterpart");
            }
            return true;
        }
        if (o->element == "film") {   // films/hdrfilm.cc:16, films/ldrfilm.cc:19
            if (t != "hdrfilm" && t != "ldrfilm") return fail(e, "film type " + t + " is not supported");
            ObjectPtr rf;
            store_.objects.get("rfilter", &rf, true);
            if (!store_.ints.get("width", &o->width, true) || !store_.ints.get("height", &o->height, true) ||
                o->width <= 0 || o->height <= 0)
                return fail(e, "needs a positive width and height");
            return true;
        }
        if (o->element == "sensor") {   // cameras/perspective.cc:23-29
            if (t != "perspective") return fail(e, "sensor type " + t + " is not supported");
            double aperture = 0.0, focus = 0.0;
            if (!store_.transforms.get("toWorld", &o->toWorld, true)) return fail(e, "needs a toWorld transform");
            store_.doubles.get("apertureRadius", &aperture, true);
            store_.doubles.get("focusDistance", &focus, true);
            if (aperture != 0.0) return fail(e, "depth of field (apertureRadius) is not supported");
            if (!store_.doubles.get("fov", &o->fov, true)) return fail(e, "needs a fov");
            if (!store_.objects.get("film", &o->film, true) || !o->film || o->film->element != "film")
                return fail(e, "needs a film");
            return true;
        }
        if (o->element == "sampler") {   // samplers/independent.cc:10: the seed is fixed
            if (t != "independent") return fail(e, "sampler type " + t + " is not supported");
            return true;
        }
        if (o->element == "rfilter") return true;   // the film's reconstruction filter: box weights
        if (o->element == "emitter") {   // lights/envmap.cc:50-54
            if (t != "envmap") return fail(e, "emitter type " + t + " is not supported");
            // worldCenter / worldRadius bound the reference's environment shadow rays; the
            // GPU path bounds them by the scene's box instead
            double sc = 1.0, radius = 2.0;
            std::string file;
            store_.doubles.get("worldRadius", &radius, true);
            if (!store_.strings.get("filename", &file, true)) return fail(e, "needs a filename");
            store_.transforms.get("toWorld", &o->toWorld, true);
            store_.doubles.get("scale", &sc, true);
            if (!o->toWorld.isIdentity()) return fail(e, "a transformed environment map is not supported");
            if (file.size() < 4 || file.compare(file.size() - 4, 4, ".hdr") != 0)
                return fail(e, "only .hdr environment maps are supported");
            if (!loadHdr(file, &o->env, &o->envW, &o->envH, &why)) return fail(e, why);
            for (auto &x : o->env) x = static_cast<float>(x * sc);
            return true;
        }
        return fail(e, "element type " + t + " is not supported");
    }

    bool shape(const XmlElem &e) {   // spica/sceneparser.cc:241-275
        const char *type = e.attr("type");
        if (!type) return fail(e, "no type");
        ObjectPtr bsdf, sub, medium;
        store_.objects.get("bsdf", &bsdf, true);
        store_.objects.get("subsurface", &sub, true);
        store_.objects.get("medium", &medium, true);
        Mat4 toWorld = Mat4::identity();
        store_.transforms.get("toWorld", &toWorld, true);
        if (sub || medium) return fail(e, "subsurface scattering and media are not supported");
        std::vector<float> tris;
        std::string why, file;
        const std::string t = type;
        if (t == "ply" || t == "obj") {
            if (!store_.strings.get("filename", &file, false)) return fail(e, "needs a filename");
            if (!(t == "ply" ? loadPly(file, toWorld, &tris, &why) : loadObj(file, toWorld, &tris, &why)))
                return fail(e, why);
        } else {
            return fail(e, "shape type " + t + " is not created by the reference's parser");
        }
        // material: the consumed bsdf, else none (a black surface)
        float rec[8] = {SPGPU_MAT_LAMBERT, 0, 0, 0, 0, 0, 0, 0};
        if (bsdf) std::memcpy(rec, bsdf->material, sizeof(rec));
        int mi = -1;
        for (size_t k = 0; k < out_->materials.size() / 8 && mi < 0; k++)
            if (std::memcmp(&out_->materials[8 * k], rec, sizeof(rec)) == 0) mi = static_cast<int>(k);
        if (mi < 0) {
            mi = static_cast<int>(out_->materials.size() / 8);
            out_->materials.insert(out_->materials.end(), rec, rec + 8);
        }
        // an area light per triangle (createPrimitive, spica/sceneparser.cc:182-190):
        // radiance read without removal (lights/area.cc:23)
        float L[3] = {0, 0, 0};
        if (waitArea_) {
            Spectrum3 r;
            if (!store_.spectra.get("radiance", &r, false)) return fail(e, "area emitter needs a radiance");
            for (int i = 0; i < 3; i++) L[i] = static_cast<float>(r.v[i]);
        }
        const size_t n = tris.size() / 9;
        out_->verts.insert(out_->verts.end(), tris.begin(), tris.end());
        for (size_t k = 0; k < n; k++) {
            out_->triMat.push_back(mi);
            out_->emit.insert(out_->emit.end(), L, L + 3);
        }
        waitArea_ = false;
        return true;
    }

    std::string file_, dir_, err_;
    Store store_;
    Loaded *out_ = nullptr;
    bool waitArea_ = false;
};

}  // namespace

extern "C" {


static int sceneLoad(const char *path, spgpu_scene_file **out);

// No C++ exception leaves the C ABI: an allocation failure or any other exception becomes
// a status and a message.
int spgpu_scene_load(const char *path, spgpu_scene_file **out) {
    try {
        return sceneLoad(path, out);
    } catch (const std::bad_alloc &) {
        setError("spgpu_scene_load: out of host memory");
        return SPGPU_ENOMEM;
    } catch (const std::exception &e) {
        setError(std::string("spgpu_scene_load: ") + e.what());
        return SPGPU_EINVAL;
    }
}

static int sceneLoad(const char *path, spgpu_scene_file **out) {
    if (!path || !out) {
        setError("spgpu_scene_load: invalid arguments");
        return SPGPU_EINVAL;
    }
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        setError(std::string("spgpu_scene_load: cannot open ") + path);
        return SPGPU_EINVAL;
    }
    const std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    XmlElem root;
    XmlReader xr(text);
    if (!xr.document(&root)) {
        setError(std::string("spgpu_scene_load: ") + path + ": " + xr.error());
        return SPGPU_EINVAL;
    }
    auto *S = new spgpu_scene_file();
    std::memset(S, 0, sizeof(*S));
    auto *data = new Loaded();
    S->internal = data;
    Parser parser(path);
    if (!parser.run(root, data)) {
        setError("spgpu_scene_load: " + parser.error());
        spgpu_scene_free(S);
        return SPGPU_EINVAL;
    }
    Loaded &L = *data;
    int spp = 0, maxDepth = 16;
    Store &st = parser.store();
    if (!st.ints.get("sampleCount", &spp, false) || spp < 0) {
        setError("spgpu_scene_load: no sampleCount (SamplerIntegrator::render reads it, core/integrator.cc:63)");
        spgpu_scene_free(S);
        return SPGPU_EINVAL;
    }
    st.ints.get("maxDepth", &maxDepth, false);
    if (L.integrator.empty()) {
        setError("spgpu_scene_load: no <integrator>");
        spgpu_scene_free(S);
        return SPGPU_EINVAL;
    }
    spgpu_scene_file &P = *S;
    P.ntri = static_cast<int32_t>(L.triMat.size());
    P.verts = L.verts.data();
    P.tri_mat = L.triMat.data();
    P.nmat = static_cast<int32_t>(L.materials.size() / 8);
    P.materials = L.materials.data();
    P.tri_emit = L.emit.data();
    P.env_width = L.envW;
    P.env_height = L.envH;
    P.env = L.env.empty() ? nullptr : L.env.data();
    // camera: eye, a point one unit along the view direction and up from the sensor's
    // toWorld (cameras/perspective.cc: camera space looks along +z with +y up)
    const Mat4 &c2w = L.camera->toWorld;
    const double o0[3] = {0, 0, 0}, z[3] = {0, 0, 1}, y[3] = {0, 1, 0};
    double eye[3], dir[3], up[3];
    c2w.point(o0, eye);
    c2w.vector(z, dir);
    c2w.vector(y, up);
    for (int i = 0; i < 3; i++) {
        P.desc.camera[i] = static_cast<float>(eye[i]);
        P.desc.camera[3 + i] = static_cast<float>(eye[i] + dir[i]);
        P.desc.camera[6 + i] = static_cast<float>(up[i]);
    }
    P.desc.camera[9] = static_cast<float>(L.camera->fov);
    P.desc.width = L.camera->film->width;
    P.desc.height = L.camera->film->height;
    P.desc.spp = spp;
    P.desc.max_depth = maxDepth;
    P.desc.integrator = L.integrator == "direct" ? SPGPU_INTEGRATOR_DIRECT : SPGPU_INTEGRATOR_PATH;
    *out = &P;
    return 0;
}

void spgpu_scene_free(spgpu_scene_file *scene) {
    if (!scene) return;
    delete static_cast<Loaded *>(scene->internal);
    delete scene;
}

int spgpu_load_hdr(const char *path, float *rgb, int32_t max_pixels, int32_t *width, int32_t *height) {
    if (!path || !width || !height) {
        setError("spgpu_load_hdr: invalid arguments");
        return SPGPU_EINVAL;
    }
    std::vector<float> px;
    int w = 0, h = 0;
    std::string why;
    bool ok;
    try {
        ok = loadHdr(path, &px, &w, &h, &why);
    } catch (const std::bad_alloc &) {
        setError("spgpu_load_hdr: out of host memory");
        return SPGPU_ENOMEM;
    }
    if (!ok) {
        setError("spgpu_load_hdr: " + why);
        return SPGPU_EINVAL;
    }
    *width = w;
    *height = h;
    if (rgb) {
        if (static_cast<int64_t>(w) * h > max_pixels) {
            setError("spgpu_load_hdr: the image has more pixels than max_pixels");
            return SPGPU_EINVAL;
        }
        std::memcpy(rgb, px.data(), px.size() * sizeof(float));
    }
    return 0;
}

}  // extern "C"
