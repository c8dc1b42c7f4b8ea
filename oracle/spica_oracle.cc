// spica_oracle.cc -- C++ restatement of the reference renderer's unidirectional
// path-tracing hot path, in double precision, behind oracle/spo_api.h.
//
// TEST INFRASTRUCTURE ONLY.  Tests, the smoke check and the benchmark's CPU
// baseline load it (oracle/_port/libspica_oracle.so); the CUDA product path never
// does.  It exists because the reference itself (oracle/_ref) can only be built
// where the reference tree is present; this restatement builds on any host, and
// its outputs are pinned against the compiled reference by tests/test_oracle.py
// (bit-identical hit primitives and distances, BSDF tables to 1e-12, renders
// sample-for-sample).
//
// Each piece follows the reference function named beside it and keeps its order
// of floating-point operations, so results match to the last bit where the same
// libm is used.  Build with -ffp-contract=off (no fused multiply-add).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "spo_api.h"

namespace spo {

static const double kPi = 4.0 * std::atan(1.0);     // core/common.h:52
static const double kInvPi = 1.0 / kPi;
static const double kInf = 1.0e32;                   // core/common.h:54
static const double kEps = 1.0e-12;                  // core/common.h:55

// ----------------------------------------------------------------------------
// vectors and RGB (core/vector3d_detail.h, core/spectrum.cc)
// ----------------------------------------------------------------------------
struct V3 {
    double x = 0, y = 0, z = 0;
    V3() = default;
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3 &a, const V3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3 &a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(const V3 &a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, const V3 &a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double absDot(const V3 &a, const V3 &b) { return std::abs(dot(a, b)); }
inline V3 cross(const V3 &a, const V3 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(const V3 &a) { return std::sqrt(dot(a, a)); }
// Vector3d::normalized / Normal3d::normalized: multiply by 1/|v|
inline V3 normalizedMul(const V3 &a) { return a * (1.0 / norm(a)); }
// vect::normalize (core/vect_math.h:38-43): divide by |v|
inline V3 normalizeDiv(const V3 &a) {
    const double n = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return {a.x / n, a.y / n, a.z / n};
}
inline V3 vmin(const V3 &a, const V3 &b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax(const V3 &a, const V3 &b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }

struct RGB {
    double r = 0, g = 0, b = 0;
    RGB() = default;
    explicit RGB(double v) : r(v), g(v), b(v) {}
    RGB(double a, double c, double d) : r(a), g(c), b(d) {}
    bool isBlack() const { return r == 0.0 && g == 0.0 && b == 0.0; }
    double gray() const { return 0.2126 * r + 0.7152 * g + 0.0722 * b; }   // spectrum.cc:677
};
inline RGB operator+(const RGB &a, const RGB &b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
inline RGB operator-(const RGB &a, const RGB &b) { return {a.r - b.r, a.g - b.g, a.b - b.b}; }
inline RGB operator*(const RGB &a, const RGB &b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
inline RGB operator*(const RGB &a, double s) { return {a.r * s, a.g * s, a.b * s}; }
inline RGB operator*(double s, const RGB &a) { return {s * a.r, s * a.g, s * a.b}; }
inline RGB operator/(const RGB &a, const RGB &b) { return {a.r / b.r, a.g / b.g, a.b / b.b}; }
inline RGB operator/(const RGB &a, double s) { return {a.r / s, a.g / s, a.b / s}; }
inline RGB rgbSqrt(const RGB &a) { return {std::sqrt(a.r), std::sqrt(a.g), std::sqrt(a.b)}; }

inline double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// core/float.h:23-47 -- one double ulp up / down
inline double nextUp(double d) {
    if (std::isinf(d) && d > 0.0) return d;
    if (d == -0.0) d = 0.0;
    uint64_t u;
    std::memcpy(&u, &d, 8);
    if (d > 0.0) u++; else u--;
    std::memcpy(&d, &u, 8);
    return d;
}
inline double nextDown(double d) {
    if (std::isinf(d) && d > 0.0) return d;
    if (d == -0.0) d = 0.0;
    uint64_t u;
    std::memcpy(&u, &d, 8);
    if (d > 0.0) u--; else u++;
    std::memcpy(&d, &u, 8);
    return d;
}

// ----------------------------------------------------------------------------
// MT19937 + Independent sampler (core/random.cc:70-163, samplers/independent.cc)
// The published Mersenne Twister (Matsumoto & Nishimura 1998), [0,1) = int32 * 2^-32.
// ----------------------------------------------------------------------------
class MT19937 {
public:
    explicit MT19937(uint32_t seed) {
        mt_[0] = seed;
        for (int i = 1; i < 624; i++) mt_[i] = 1812433253u * (mt_[i - 1] ^ (mt_[i - 1] >> 30)) + (uint32_t)i;
        idx_ = 624;
    }
    uint32_t next() {
        if (idx_ >= 624) twist();
        uint32_t y = mt_[idx_++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        return y;
    }
    double get1D() { return next() * (1.0 / 4294967296.0); }

private:
    void twist() {
        for (int k = 0; k < 624; k++) {
            const uint32_t y = (mt_[k] & 0x80000000u) | (mt_[(k + 1) % 624] & 0x7fffffffu);
            mt_[k] = mt_[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        idx_ = 0;
    }
    uint32_t mt_[624];
    int idx_;
};

struct P2 {
    double u0, u1;
};
struct Sampler {
    MT19937 rng;
    explicit Sampler(uint32_t s) : rng(s) {}
    double get1D() { return rng.get1D(); }
    P2 get2D() {   // Sampler::get2D: Point2d{get1D(), get1D()} (evaluation in order)
        const double a = get1D();
        const double b = get1D();
        return {a, b};
    }
};

// ----------------------------------------------------------------------------
// 4x4 transforms, enough for the perspective camera (core/transform.cc,
// core/matrix4x4.cc).  Inverse by Gauss-Jordan elimination with full pivoting.
// ----------------------------------------------------------------------------
struct M4 {
    double m[4][4];
    static M4 identity() {
        M4 r{};
        for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r.m[i][j] = i == j ? 1.0 : 0.0;
        return r;
    }
};
inline M4 mul(const M4 &a, const M4 &b) {
    M4 r{};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            r.m[i][j] = 0.0;
            for (int k = 0; k < 4; k++) r.m[i][j] += a.m[i][k] * b.m[k][j];
        }
    return r;
}
inline M4 inverse(const M4 &a) {
    int indxc[4], indxr[4];
    int ipiv[4] = {0, 0, 0, 0};
    double v[4][4];
    std::memcpy(v, a.m, sizeof(v));
    for (int i = 0; i < 4; i++) {
        int irow = 0, icol = 0;
        double big = 0.0;
        for (int j = 0; j < 4; j++) {
            if (ipiv[j] == 1) continue;
            for (int k = 0; k < 4; k++) {
                if (ipiv[k] == 0 && std::abs(v[j][k]) >= big) {
                    big = std::abs(v[j][k]);
                    irow = j;
                    icol = k;
                }
            }
        }
        ++ipiv[icol];
        if (irow != icol) for (int k = 0; k < 4; k++) std::swap(v[irow][k], v[icol][k]);
        indxr[i] = irow;
        indxc[i] = icol;
        const double pinv = 1.0 / v[icol][icol];
        v[icol][icol] = 1.0;
        for (int j = 0; j < 4; j++) v[icol][j] *= pinv;
        for (int j = 0; j < 4; j++) {
            if (j == icol) continue;
            const double save = v[j][icol];
            v[j][icol] = 0.0;
            for (int k = 0; k < 4; k++) v[j][k] -= v[icol][k] * save;
        }
    }
    for (int j = 3; j >= 0; j--)
        if (indxr[j] != indxc[j])
            for (int k = 0; k < 4; k++) std::swap(v[k][indxr[j]], v[k][indxc[j]]);
    M4 r;
    std::memcpy(r.m, v, sizeof(v));
    return r;
}
struct Xf {   // a transform with its inverse, composed as in Transform::operator*=
    M4 m, inv;
    static Xf fromMatrix(const M4 &a) { return {a, inverse(a)}; }
    Xf inverted() const { return {inv, m}; }
};
inline Xf compose(const Xf &a, const Xf &b) { return {mul(a.m, b.m), mul(b.inv, a.inv)}; }
inline Xf scaleXf(double sx, double sy, double sz) {
    M4 m = M4::identity(), i = M4::identity();
    m.m[0][0] = sx; m.m[1][1] = sy; m.m[2][2] = sz;
    i.m[0][0] = 1.0 / sx; i.m[1][1] = 1.0 / sy; i.m[2][2] = 1.0 / sz;
    return {m, i};
}
inline Xf translateXf(const V3 &d) {
    M4 m = M4::identity(), i = M4::identity();
    m.m[0][3] = d.x; m.m[1][3] = d.y; m.m[2][3] = d.z;
    i.m[0][3] = -d.x; i.m[1][3] = -d.y; i.m[2][3] = -d.z;
    return {m, i};
}
inline V3 applyPoint(const M4 &m, const V3 &p) {   // Transform::apply(Point3d), transform.cc:60
    const double ps[4] = {p.x, p.y, p.z, 1.0};
    double r[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r[i] += m.m[i][j] * ps[j];
    if (r[3] != 1.0) {
        r[0] /= (r[3] + kEps);
        r[1] /= (r[3] + kEps);
        r[2] /= (r[3] + kEps);
    }
    return {r[0], r[1], r[2]};
}
inline V3 applyVector(const M4 &m, const V3 &v) {   // transform.cc:85
    return {m.m[0][0] * v.x + m.m[0][1] * v.y + m.m[0][2] * v.z,
            m.m[1][0] * v.x + m.m[1][1] * v.y + m.m[1][2] * v.z,
            m.m[2][0] * v.x + m.m[2][1] * v.y + m.m[2][2] * v.z};
}

struct Camera {   // PerspectiveCamera, cameras/perspective.cc:36-74; Camera, core/camera.cc:20-38
    Xf cameraToWorld, rasterToCamera;
    Camera(const double *c, int W, int H) {
        const V3 eye(c[0], c[1], c[2]), look(c[3], c[4], c[5]), up(c[6], c[7], c[8]);
        // Transform::lookAt (transform.cc:167)
        M4 c2w{};
        c2w.m[0][3] = eye.x; c2w.m[1][3] = eye.y; c2w.m[2][3] = eye.z; c2w.m[3][3] = 1.0;
        const V3 dir = normalizedMul(look - eye);
        V3 left = cross(normalizedMul(up), dir);
        left = normalizedMul(left);
        const V3 newUp = cross(dir, left);
        c2w.m[0][0] = left.x; c2w.m[1][0] = left.y; c2w.m[2][0] = left.z;
        c2w.m[0][1] = newUp.x; c2w.m[1][1] = newUp.y; c2w.m[2][1] = newUp.z;
        c2w.m[0][2] = dir.x; c2w.m[1][2] = dir.y; c2w.m[2][2] = dir.z;
        cameraToWorld = Xf::fromMatrix(c2w);
        // Transform::perspective (transform.cc:205)
        const double fov = c[9] * kPi / 180.0;
        const double aspect = static_cast<double>(W) / H;
        const double n = 1.0e-2, f = 1000.0;
        M4 pers{};
        pers.m[0][0] = 1.0 / aspect; pers.m[1][1] = 1.0;
        pers.m[2][2] = f / (f - n); pers.m[2][3] = -f * n / (f - n);
        pers.m[3][2] = 1.0;
        const double invTanHalf = 1.0 / std::tan(fov / 2.0);
        const Xf cameraToScreen = compose(scaleXf(invTanHalf, invTanHalf, 1.0), Xf::fromMatrix(pers));
        // screen window [-1,1]^2
        const Xf screenToRaster = compose(compose(scaleXf(W, H, 1.0), scaleXf(1.0 / 2.0, -1.0 / 2.0, 1.0)),
                                          translateXf(V3(1.0, -1.0, 0.0)));
        const Xf rasterToScreen = screenToRaster.inverted();
        rasterToCamera = compose(cameraToScreen.inverted(), rasterToScreen);
    }
    void spawnRay(int px, int py, P2 film, V3 *org, V3 *dir) const {
        const V3 pFilm(px + film.u0, py + film.u1, 0.0);
        const V3 pCamera = applyPoint(rasterToCamera.m, pFilm);
        const V3 d = normalizeDiv(pCamera);   // pinhole (lensRadius 0): the lens sample is unused
        *org = applyPoint(cameraToWorld.m, V3(0.0, 0.0, 0.0));
        *dir = applyVector(cameraToWorld.m, d);
    }
};

// ----------------------------------------------------------------------------
// rays, triangles, bounds (core/ray.cc, core/triangle.cc, core/bounds3d_detail.h)
// ----------------------------------------------------------------------------
struct Ray {
    V3 o, d, inv;
    double maxDist;
    Ray(const V3 &org, const V3 &dir, double tmax = kInf) : o(org), d(normalizedMul(dir)), maxDist(tmax) {
        inv.x = d.x == 0.0 ? kInf : 1.0 / d.x;
        inv.y = d.y == 0.0 ? kInf : 1.0 / d.y;
        inv.z = d.z == 0.0 ? kInf : 1.0 / d.z;
    }
};

struct Box {
    V3 lo{std::numeric_limits<double>::max(), std::numeric_limits<double>::max(), std::numeric_limits<double>::max()};
    V3 hi{std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest()};
    void merge(const Box &b) { lo = vmin(lo, b.lo); hi = vmax(hi, b.hi); }
    void merge(const V3 &p) { lo = vmin(p, lo); hi = vmax(p, hi); }
    double area() const {
        const V3 df = hi - lo;
        const double xy = std::abs(df.x * df.y), yz = std::abs(df.y * df.z), zx = std::abs(df.z * df.x);
        return 2.0 * (xy + yz + zx);
    }
    int maxExtent() const {
        const V3 df = hi - lo;
        if (df.x >= df.y && df.x >= df.z) return 0;
        if (df.y >= df.z) return 1;
        return 2;
    }
    bool hit(const Ray &r, double *tNear = nullptr, double *tFar = nullptr) const {   // bounds3d_detail.h:64
        double t0 = 0.0, t1 = r.maxDist;
        for (int i = 0; i < 3; i++) {
            double a = (lo[i] - r.o[i]) * r.inv[i];
            double b = (hi[i] - r.o[i]) * r.inv[i];
            if (a > b) std::swap(a, b);
            t0 = std::max(t0, a);
            t1 = std::min(t1, b);
            if (t0 > t1) return false;
        }
        if (tNear) *tNear = t0;
        if (tFar) *tFar = t1;
        return true;
    }
};
inline Box merged(const Box &a, const Box &b) {
    Box r;
    r.lo = vmin(a.lo, b.lo);
    r.hi = vmax(a.hi, b.hi);
    return r;
}

struct Tri {
    V3 p[3];
    V3 n;   // face normal, triangle.cc:28-29
};

struct Hit {   // the parts of SurfaceInteraction the path uses
    V3 pos, n, dpdu, dpdv, wo;
    int prim = -1;
};

// coordinateSystem (core/vect_math.h:116)
inline void coordSystem(const V3 &w, V3 *u, V3 *v) {
    if (std::abs(w.x) > std::abs(w.y)) *u = normalizeDiv(V3(-w.z, 0, w.x));
    else *u = normalizeDiv(V3(0, w.z, -w.y));
    *v = normalizeDiv(cross(w, *u));
}

// Triangle::intersect, triangle.cc:98-157 (closest, fills the hit) and :159-178
inline bool triHit(const Tri &T, const Ray &r, double *tHit, double *uu, double *vv) {
    const V3 e1 = T.p[1] - T.p[0], e2 = T.p[2] - T.p[0];
    const V3 pv = cross(r.d, e2);
    const double det = dot(e1, pv);
    if (det > -kEps && det < kEps) return false;
    const double invdet = 1.0 / det;
    const V3 tv = r.o - T.p[0];
    const double u = dot(tv, pv) * invdet;
    if (u < 0.0 || u > 1.0) return false;
    const V3 qv = cross(tv, e1);
    const double v = dot(r.d, qv) * invdet;
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = dot(e2, qv) * invdet;
    if (t <= kEps || t > r.maxDist) return false;
    *tHit = t;
    if (uu) *uu = u;
    if (vv) *vv = v;
    return true;
}
inline void fillHit(const Tri &T, const Ray &r, double t, Hit *h) {
    h->pos = r.o + t * r.d;
    coordSystem(T.n, &h->dpdu, &h->dpdv);   // the scenes carry no uvs: detUV == 0
    h->n = normalizeDiv(cross(h->dpdu, h->dpdv));
    h->wo = -r.d;
    // shading normal equals the face normal (flat triangles): no shading frame change
}
inline double triArea(const Tri &T) { return 0.5 * norm(cross(T.p[1] - T.p[0], T.p[2] - T.p[0])); }

// offsetRayOrigin (core/interaction.cc:16)
inline V3 offsetOrigin(const V3 &p, const V3 &n, const V3 &w) {
    V3 off = n * 1.0e-3;
    if (dot(w, n) < 0.0) off = -off;
    const V3 po = p + off;
    double r[3];
    for (int i = 0; i < 3; i++) r[i] = off[i] > 0.0 ? nextUp(po[i]) : nextDown(po[i]);
    return {r[0], r[1], r[2]};
}
inline Ray spawnRay(const V3 &p, const V3 &n, const V3 &w) { return Ray(offsetOrigin(p, n, w), w, kInf); }
inline Ray spawnRayTo(const V3 &p1, const V3 &n1, const V3 &p2, const V3 &n2) {   // interaction.cc:88
    const V3 o = offsetOrigin(p1, n1, p2 - p1);
    const V3 tgt = offsetOrigin(p2, n2, o - p2);
    const V3 d = tgt - o;
    return Ray(o, d, norm(d));
}

// ----------------------------------------------------------------------------
// binary BVH (accelerators/bvh.cc:139-237, :331-387)
// ----------------------------------------------------------------------------
struct PrimInfo {
    int prim;
    V3 centroid;
    Box bounds;
};
struct Node {
    Box bounds;
    int left = -1, right = -1, prim = -1;
};

class BVH {
public:
    void build(const std::vector<Tri> &tris) {
        tris_ = &tris;
        nodes_.clear();
        if (tris.empty()) return;
        std::vector<PrimInfo> info(tris.size());
        for (size_t i = 0; i < tris.size(); i++) {
            Box b;
            const Tri &T = tris[i];
            b.lo = vmin(T.p[0], vmin(T.p[1], T.p[2]));
            b.hi = vmax(T.p[0], vmax(T.p[1], T.p[2]));
            info[i] = {static_cast<int>(i), (b.hi + b.lo) * 0.5, b};
        }
        nodes_.reserve(2 * tris.size());
        rec(info, 0, static_cast<int>(tris.size()));
    }

    bool closest(Ray &r, Hit *h) const {
        if (nodes_.empty()) return false;
        std::vector<int> &st = stack();
        st.clear();
        st.push_back(0);
        bool found = false;
        while (!st.empty()) {
            const Node &nd = nodes_[st.back()];
            st.pop_back();
            if (nd.prim >= 0) {
                double t;
                if (triHit((*tris_)[nd.prim], r, &t, nullptr, nullptr)) {
                    r.maxDist = t;   // GeometricPrimitive::intersect, primitive.cc:52
                    h->prim = nd.prim;
                    fillHit((*tris_)[nd.prim], r, t, h);
                    found = true;
                }
            } else if (nd.bounds.hit(r)) {
                if (nd.left >= 0) st.push_back(nd.left);
                if (nd.right >= 0) st.push_back(nd.right);
            }
        }
        return found;
    }

    bool any(const Ray &r) const {
        if (nodes_.empty()) return false;
        std::vector<int> &st = stack();
        st.clear();
        st.push_back(0);
        while (!st.empty()) {
            const Node &nd = nodes_[st.back()];
            st.pop_back();
            if (nd.prim >= 0) {
                double t;
                if (triHit((*tris_)[nd.prim], r, &t, nullptr, nullptr)) return true;
            } else if (nd.bounds.hit(r)) {
                if (nd.left >= 0) st.push_back(nd.left);
                if (nd.right >= 0) st.push_back(nd.right);
            }
        }
        return false;
    }

private:
    static std::vector<int> &stack() {
        thread_local std::vector<int> s;
        return s;
    }

    int rec(std::vector<PrimInfo> &data, int start, int end) {
        if (start == end) return -1;
        const int id = static_cast<int>(nodes_.size());
        nodes_.emplace_back();
        Box bounds;
        for (int i = start; i < end; i++) bounds = merged(bounds, data[i].bounds);
        const int n = end - start;
        if (n == 1) {
            nodes_[id].bounds = bounds;
            nodes_[id].prim = data[start].prim;
            return id;
        }
        Box cb;
        for (int i = start; i < end; i++) cb.merge(data[i].centroid);
        const int axis = cb.maxExtent();
        int mid = (start + end) / 2;
        if (n <= 8) {
            std::nth_element(data.begin() + start, data.begin() + mid, data.begin() + end,
                             [axis](const PrimInfo &a, const PrimInfo &b) {
                                 return a.centroid[axis] < b.centroid[axis];
                             });
        } else {
            const int nb = 16;
            int count[nb] = {0};
            Box bb[nb];
            const double cmin = cb.lo[axis], cmax = cb.hi[axis];
            const double idenom = 1.0 / (std::abs(cmax - cmin) + kEps);
            for (int i = start; i < end; i++) {
                const double num = data[i].centroid[axis] - cb.lo[axis];
                int b = static_cast<int>(nb * std::abs(num) * idenom);
                if (b == nb) b = nb - 1;
                count[b]++;
                bb[b] = merged(bb[b], data[i].bounds);
            }
            double cost[nb - 1] = {0};
            for (int i = 0; i < nb - 1; i++) {
                Box b0, b1;
                int c0 = 0, c1 = 0;
                for (int j = 0; j <= i; j++) { b0 = merged(b0, bb[j]); c0 += count[j]; }
                for (int j = i + 1; j < nb; j++) { b1 = merged(b1, bb[j]); c1 += count[j]; }
                cost[i] += 0.125 + (c0 * b0.area() + c1 * b1.area()) / bounds.area();
            }
            double minCost = cost[0];
            int split = 0;
            for (int i = 1; i < nb - 1; i++) {
                if (minCost > cost[i]) { minCost = cost[i]; split = i; }
            }
            if (minCost < n) {
                auto it = std::partition(data.begin() + start, data.begin() + end,
                                         [&](const PrimInfo &p) {
                                             const double inv = 1.0 / (std::abs(cmax - cmin) + kEps);
                                             const double diff = std::abs(p.centroid[axis] - cmin);
                                             int b = static_cast<int>(nb * diff * inv);
                                             if (b >= nb) b = nb - 1;
                                             return b <= split;
                                         });
                mid = static_cast<int>(it - data.begin());
            }
        }
        const int l = rec(data, start, mid);
        const int r = rec(data, mid, end);
        nodes_[id].bounds = bounds;
        nodes_[id].left = l;
        nodes_[id].right = r;
        return id;
    }

    const std::vector<Tri> *tris_ = nullptr;
    std::vector<Node> nodes_;
};

// ----------------------------------------------------------------------------
// environment map: MipMap (core/mipmap.cc) + Distribution1D/2D (core/sampling.cc)
// ----------------------------------------------------------------------------
struct Image {
    int w = 0, h = 0;
    std::vector<RGB> px;
    const RGB &at(int x, int y) const { return px[static_cast<size_t>(y) * w + x]; }
};

class MipMap {
public:
    void init(const Image &img) {
        levels_.clear();
        int nLevels = 1;
        for (int v = std::max(img.w, img.h); v != 0; v >>= 1) nLevels++;   // 1 + log2Int
        levels_.resize(nLevels);
        levels_[0] = img;
        for (int i = 1; i < nLevels; i++) {
            Image &L = levels_[i];
            L.w = std::max(1, levels_[i - 1].w / 2);
            L.h = std::max(1, levels_[i - 1].h / 2);
            L.px.resize(static_cast<size_t>(L.w) * L.h);
            for (int y = 0; y < L.h; y++)
                for (int x = 0; x < L.w; x++)
                    L.px[static_cast<size_t>(y) * L.w + x] =
                        0.25 * (texel(i - 1, 2 * x, 2 * y) + texel(i - 1, 2 * x + 1, 2 * y) +
                                texel(i - 1, 2 * x, 2 * y + 1) + texel(i - 1, 2 * x + 1, 2 * y + 1));
        }
    }
    int levels() const { return static_cast<int>(levels_.size()); }
    RGB texel(int level, int s, int t) const {   // ImageWrap::Repeat
        const int w = levels_[level].w, h = levels_[level].h;
        s = (s % w + w) % w;
        t = (t % h + h) % h;
        return levels_[level].at(s, t);
    }
    RGB bilinear(int level, double s0, double t0) const {
        level = std::max(0, std::min(level, levels()));
        const double s = s0 * levels_[level].w - 0.5;
        const double t = t0 * levels_[level].h - 0.5;
        const int si = static_cast<int>(s), ti = static_cast<int>(t);
        const double ds = s - si, dt = t - ti;
        return (1.0 - ds) * (1.0 - dt) * texel(level, si, ti) + ds * (1.0 - dt) * texel(level, si + 1, ti) +
               (1.0 - ds) * dt * texel(level, si, ti + 1) + ds * dt * texel(level, si + 1, ti + 1);
    }
    RGB lookup(double s, double t, double width = 0.0) const {   // mipmap.cc:67
        const double level = levels() - 1 + std::log2(std::max(width, 1.0e-8));
        if (level < 0) return bilinear(0, s, t);
        if (level >= levels() - 1) return texel(levels() - 1, 0, 0);
        const int l = static_cast<int>(level);
        const double delta = level - l;
        return (1.0 - delta) * bilinear(static_cast<int>(level), s, t) +
               delta * bilinear(static_cast<int>(level + 1), s, t);
    }

private:
    std::vector<Image> levels_;
};

class Dist1D {
public:
    Dist1D() = default;
    explicit Dist1D(const std::vector<double> &f) : func_(f) {
        const int n = static_cast<int>(f.size());
        cdf_.assign(n + 1, 0.0);
        for (int i = 1; i < n + 1; i++) cdf_[i] = cdf_[i - 1] + func_[i - 1] / n;
        integral_ = cdf_[n];
        if (integral_ == 0.0) {
            for (int i = 1; i < n + 1; i++) cdf_[i] = static_cast<double>(i) / n;
        } else {
            for (int i = 1; i < n + 1; i++) cdf_[i] /= integral_;
        }
    }
    int count() const { return static_cast<int>(func_.size()); }
    double integral() const { return integral_; }
    double func(int i) const { return func_[i]; }
    double sample(double u, double *pdf, int *offset) const {
        int off = static_cast<int>(std::upper_bound(cdf_.begin(), cdf_.end(), u) - cdf_.begin()) - 1;
        off = std::min(off, static_cast<int>(cdf_.size()) - 1);
        if (offset) *offset = off;
        double du = u - cdf_[off];
        if (cdf_[off + 1] - cdf_[off] > 0.0) du /= (cdf_[off + 1] - cdf_[off]);
        *pdf = func_[off] / integral_;
        return (off + du) / func_.size();
    }

private:
    std::vector<double> func_, cdf_;
    double integral_ = 0.0;
};

struct Envmap {   // lights/envmap.cc with an identity toWorld
    MipMap mip;
    std::vector<Dist1D> cond;
    Dist1D marg;
    V3 center;
    double radius = 0.0;

    void init(const Image &img, const V3 &c, double r) {
        center = c;
        radius = r;
        mip.init(img);   // scale 1.0
        const int w = img.w, h = img.h;
        const double filter = 1.0 / std::max(w, h);
        std::vector<double> row(w), margF(h);
        cond.clear();
        for (int v = 0; v < h; v++) {
            const double vp = static_cast<double>(v + 0.5) / h;
            const double sinTheta = std::sin(kPi * (v + 0.5) / h);
            for (int u = 0; u < w; u++) {
                const double up = static_cast<double>(u + 0.5) / w;
                row[u] = mip.lookup(up, vp, filter).gray();
                row[u] *= sinTheta;
            }
            cond.emplace_back(row);
        }
        for (int v = 0; v < h; v++) margF[v] = cond[v].integral();
        marg = Dist1D(margF);
    }
    double pdf2(double u, double v) const {   // Distribution2D::pdf
        const int iu = std::max(0, std::min(static_cast<int>(u * cond[0].count()), cond[0].count() - 1));
        const int iv = std::max(0, std::min(static_cast<int>(v * marg.count()), marg.count() - 1));
        return cond[iv].func(iu) / marg.integral();
    }
    RGB Le(const V3 &dirRaw) const {   // Envmap::Le, envmap.cc:130
        const V3 d = normalizedMul(dirRaw);
        double phi = std::atan2(d.y, d.x);
        if (phi < 0.0) phi += 2.0 * kPi;
        const double theta = std::acos(clampd(d.z, -1.0, 1.0));
        return mip.lookup(phi * (0.5 * kInvPi), theta * kInvPi);
    }
    double pdfLi(const V3 &d) const {   // envmap.cc:81
        const double theta = std::acos(clampd(d.z, -1.0, 1.0));
        double phi = std::atan2(d.y, d.x);
        if (phi < 0.0) phi += 2.0 * kPi;
        const double sinTheta = std::sin(theta);
        if (sinTheta == 0.0) return 0.0;
        return pdf2(phi * (0.5 * kInvPi), theta * kInvPi) / (2.0 * kPi * kPi * sinTheta);
    }
};

// ----------------------------------------------------------------------------
// BSDFs (core/bsdf.cc, core/bxdf.cc, core/microfacet.cc, core/fresnel.cc)
// ----------------------------------------------------------------------------
enum : int { kReflection = 1, kTransmission = 2, kDiffuse = 4, kGlossy = 8, kSpecular = 16, kAll = 31 };

inline double cosT(const V3 &w) { return w.z; }
inline double cos2T(const V3 &w) { return w.z * w.z; }
inline double sin2T(const V3 &w) { return std::max(0.0, 1.0 - cos2T(w)); }
inline double sinT(const V3 &w) { return std::sqrt(sin2T(w)); }
inline double tanT(const V3 &w) { return sinT(w) / (cosT(w) + kEps); }
inline double tan2T(const V3 &w) { return sin2T(w) / (cos2T(w) + kEps); }
inline double cosP(const V3 &w) {
    const double s = sinT(w);
    return s == 0.0 ? 1.0 : clampd(w.x / s, -1.0, 1.0);
}
inline double sinP(const V3 &w) {
    const double s = sinT(w);
    return s == 0.0 ? 0.0 : clampd(w.y / s, -1.0, 1.0);
}
inline double cos2P(const V3 &w) { const double c = cosP(w); return c * c; }
inline double sin2P(const V3 &w) { const double s = sinP(w); return s * s; }
inline bool sameHemi(const V3 &a, const V3 &b) { return a.z * b.z > 0.0; }
inline V3 reflectV(const V3 &wo, const V3 &n) { return -wo + n * 2.0 * dot(n, wo); }
inline bool refractV(const V3 &wi, const V3 &n, double eta, V3 *wt) {
    const double cI = dot(n, wi);
    const double s2I = std::max(0.0, 1.0 - cI * cI);
    const double s2T = eta * eta * s2I;
    if (s2T >= 1.0) return false;
    const double cT = std::sqrt(1.0 - s2T);
    *wt = eta * (-wi) + (eta * cI - cT) * n;
    return true;
}
inline V3 faceForward(const V3 &n, const V3 &v) { return dot(n, v) < 0.0 ? -n : n; }

// concentric disk + cosine hemisphere, sampling.cc:151-179
inline void concentricDisk(P2 u, double *dx, double *dy) {
    const double ox = 2.0 * u.u0 - 1.0, oy = 2.0 * u.u1 - 1.0;
    if (ox == 0.0 && oy == 0.0) { *dx = 0.0; *dy = 0.0; return; }
    double theta, r;
    if (std::abs(ox) > std::abs(oy)) {
        r = ox;
        theta = kPi * (oy / ox) / 4.0;
    } else {
        r = oy;
        theta = (kPi / 2.0) - kPi * (ox / oy) / 4.0;
    }
    *dx = r * std::cos(theta);
    *dy = r * std::sin(theta);
}
inline V3 cosineHemisphere(P2 u) {
    double x, y;
    concentricDisk(u, &x, &y);
    return {x, y, std::sqrt(std::max(0.0, 1.0 - x * x - y * y))};
}

inline double frDielectric(double cI, double etaI, double etaT) {   // fresnel.cc:65
    cI = clampd(cI, -1.0, 1.0);
    if (!(cI > 0.0)) {
        std::swap(etaI, etaT);
        cI = std::abs(cI);
    }
    const double sI = std::sqrt(std::max(0.0, 1.0 - cI * cI));
    const double sT = etaI / etaT * sI;
    if (sT >= 1.0) return 1.0;
    const double cT = std::sqrt(std::max(0.0, 1.0 - sT * sT));
    const double Rpar = ((etaT * cI) - (etaI * cT)) / ((etaT * cI) + (etaI * cT));
    const double Rperp = ((etaI * cI) - (etaT * cT)) / ((etaI * cI) + (etaT * cT));
    return 0.5 * (Rpar * Rpar + Rperp * Rperp);
}
inline RGB frConductor(double cI, const RGB &etaI, const RGB &etaT, const RGB &k) {   // fresnel.cc:40
    cI = clampd(cI, -1.0, 1.0);
    const RGB eta = etaT / etaI, etaK = k / etaI;
    const double c2 = cI * cI, s2 = 1.0 - c2;
    const RGB eta2 = eta * eta, etaK2 = etaK * etaK;
    const RGB t0 = eta2 - etaK2 - RGB(s2);
    const RGB a2b2 = rgbSqrt(t0 * t0 + 4.0 * eta2 * etaK2);
    const RGB t1 = a2b2 + RGB(c2);
    const RGB a = rgbSqrt(0.5 * (a2b2 + t0));
    const RGB t2 = 2.0 * cI * a;
    const RGB Rs = (t1 - t2) / (t1 + t2);
    const RGB t3 = c2 * a2b2 + RGB(s2 * s2);
    const RGB t4 = t2 * s2;
    const RGB Rp = Rs * (t3 - t4) / (t3 + t4 + RGB(kEps));
    return 0.5 * (Rp + Rs);
}

struct GGX {   // TrowbridgeReitzDistribution, visible-normal sampling on
    double ax, ay;
    double D(const V3 &wh) const {
        const double t2 = tan2T(wh);
        if (std::isinf(t2)) return 0.0;
        const double c4 = cos2T(wh) * cos2T(wh);
        const double e = (cos2P(wh) / (ax * ax) + sin2P(wh) / (ay * ay)) * t2;
        return 1.0 / (kPi * ax * ay * c4 * (1.0 + e) * (1.0 + e));
    }
    double lambda(const V3 &w) const {
        const double at = std::abs(tanT(w));
        if (std::isinf(at)) return 0.0;
        const double alpha = std::sqrt(cos2P(w) * ax * ax + sin2P(w) * ay * ay);
        const double aInv = alpha * at;
        const double sgn = aInv >= 0.0 ? 1.0 : -1.0;
        return (-1.0 + sgn * std::sqrt(1.0 + aInv * aInv)) / 2.0;
    }
    double G1(const V3 &w, const V3 &wh) const {
        if (w.z * dot(w, wh) <= 0.0) return 0.0;
        return 1.0 / (1.0 + lambda(w));
    }
    double G(const V3 &wo, const V3 &wi, const V3 &wh) const {
        if (wi.z * dot(wi, wh) <= 0.0) return 0.0;
        if (wo.z * dot(wo, wh) <= 0.0) return 0.0;
        return 1.0 / (1.0 + lambda(wo) + lambda(wi));
    }
    double pdf(const V3 &wo, const V3 &wh) const {
        return D(wh) * G1(wo, wh) * absDot(wo, wh) / std::abs(cosT(wo));
    }
    // Visible-normal sampling of Heitz & d'Eon (2014): stretch, sample the slopes of
    // the alpha=1 distribution, rotate, unstretch (microfacet.cc:15-85).
    static void sample11(double cosTheta, P2 u, double *sx, double *sy) {
        if (cosTheta > 0.9999) {
            const double r = std::sqrt(u.u0 / (1.0 - u.u0));
            const double phi = 2.0 * kPi * u.u1;
            *sx = r * std::cos(phi);
            *sy = r * std::sin(phi);
            return;
        }
        const double sinTheta = std::sqrt(std::max(0.0, 1.0 - cosTheta * cosTheta));
        const double tanTheta = sinTheta / cosTheta;
        const double a = 1.0 / tanTheta;
        const double G1 = 2.0 / (1.0 + std::sqrt(1.0 + 1.0 / (a * a)));
        const double A = 2.0 * u.u0 / G1 - 1.0;
        double tmp = 1.0 / (A * A - 1.0);
        if (tmp > 1.0e10) tmp = 1.0e10;
        const double B = tanTheta;
        const double Dd = std::sqrt(std::max(0.0, B * B * tmp * tmp - (A * A - B * B) * tmp));
        const double x1 = B * tmp - Dd, x2 = B * tmp + Dd;
        *sx = (A < 0.0 || x2 > 1.0 / tanTheta) ? x1 : x2;
        double S, U;
        if (u.u1 > 0.5) { S = 1.0; U = 2.0 * (u.u1 - 0.5); }
        else { S = -1.0; U = 2.0 * (0.5 - u.u1); }
        const double z = (U * (U * (U * 0.27385 - 0.73369) + 0.46341)) /
                         (U * (U * (U * 0.093073 + 0.309420) - 1.0) + 0.597999);
        *sy = S * z * std::sqrt(1.0 + (*sx) * (*sx));
    }
    V3 sampleVis(const V3 &wi, P2 u) const {
        const V3 ws = normalizedMul(V3(ax * wi.x, ay * wi.y, wi.z));
        double sx, sy;
        sample11(cosT(ws), u, &sx, &sy);
        const double cp = cosP(ws), sp = sinP(ws);
        const double tmp = cp * sx - sp * sy;
        sy = sp * sx + cp * sy;
        sx = tmp;
        sx = sx * ax;
        sy = sy * ay;
        return normalizedMul(V3(-sx, -sy, 1.0));
    }
    V3 sample(const V3 &wo, P2 u) const {
        const bool flip = wo.z < 0.0;
        V3 wh = sampleVis(flip ? -wo : wo, u);
        if (flip) wh = -wh;
        return wh;
    }
};

// The reference's own erf / erfinv (core/math.h:14-67): Giles' single-precision
// polynomial for erfinv and Abramowitz & Stegun 7.1.26 for erf, with their float-rounded
// coefficients promoted to double as in the reference.
inline double refErfinv(double x) {
    double w, p;
    x = clampd(x, -0.99999, 0.99999);
    w = -std::log((1 - x) * (1 + x));
    if (w < 5) {
        w = w - 2.5f;
        p = 2.81022636e-08f;
        p = 3.43273939e-07f + p * w;
        p = -3.5233877e-06f + p * w;
        p = -4.39150654e-06f + p * w;
        p = 0.00021858087f + p * w;
        p = -0.00125372503f + p * w;
        p = -0.00417768164f + p * w;
        p = 0.246640727f + p * w;
        p = 1.50140941f + p * w;
    } else {
        w = std::sqrt(w) - 3;
        p = -0.000200214257f;
        p = 0.000100950558f + p * w;
        p = 0.00134934322f + p * w;
        p = -0.00367342844f + p * w;
        p = 0.00573950773f + p * w;
        p = -0.0076224613f + p * w;
        p = 0.00943887047f + p * w;
        p = 1.00167406f + p * w;
        p = 2.83297682f + p * w;
    }
    return p * x;
}
inline double refErf(double x) {
    const double a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f, a4 = -1.453152027f,
                 a5 = 1.061405429f, pp = 0.3275911f;
    int sign = 1;
    if (x < 0) sign = -1;
    x = std::abs(x);
    const double t = 1 / (1 + pp * x);
    const double y = 1 - (((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * std::exp(-x * x);
    return sign * y;
}

// BeckmannDistribution with visible-normal sampling (microfacet.cc:79-150, 273-356):
// Jakob's bisection / Newton inversion of the slope CDF.
struct Beckmann {
    double ax, ay;
    double D(const V3 &wh) const {
        const double t2 = tan2T(wh);
        if (std::isinf(t2)) return 0.0;
        const double c4 = cos2T(wh) * cos2T(wh);
        const double ab2 = cos2P(wh) / (ax * ax) + sin2P(wh) / (ay * ay);
        return std::exp(-t2 * ab2) / (kPi * ax * ay * c4);
    }
    double lambda(const V3 &w) const {
        const double at = std::abs(tanT(w));
        if (std::isinf(at)) return 0.0;
        const double alpha = std::sqrt(cos2P(w) * ax * ax + sin2P(w) * ay * ay);
        const double a = 1.0 / (alpha * at);
        if (a >= 1.6) return 0.0;
        return (1.0 - 1.259 * a + 0.396 * a * a) / (3.535 * a + 2.181 * a * a);
    }
    double G1(const V3 &w, const V3 &wh) const {
        if (w.z * dot(w, wh) <= 0.0) return 0.0;
        return 1.0 / (1.0 + lambda(w));
    }
    double G(const V3 &wo, const V3 &wi, const V3 &wh) const {
        if (wi.z * dot(wi, wh) <= 0.0) return 0.0;
        if (wo.z * dot(wo, wh) <= 0.0) return 0.0;
        return 1.0 / (1.0 + lambda(wo) + lambda(wi));
    }
    double pdf(const V3 &wo, const V3 &wh) const {
        return D(wh) * G1(wo, wh) * absDot(wo, wh) / std::abs(cosT(wo));
    }
    static void sample11(double cosThetaI, double U1, double U2, double *sx, double *sy) {
        if (cosThetaI > 0.9999) {
            const double r = std::sqrt(-std::log(1.0 - U1));
            const double sinPhi = std::sin(2.0 * kPi * U2);
            const double cosPhi = std::cos(2.0 * kPi * U2);
            *sx = r * cosPhi;
            *sy = r * sinPhi;
            return;
        }
        const double sinThetaI = std::sqrt(std::max(0.0, 1.0 - cosThetaI * cosThetaI));
        const double tanThetaI = sinThetaI / cosThetaI;
        const double cotThetaI = 1.0 / tanThetaI;
        double a = -1.0;
        double c = refErf(cotThetaI);
        const double samplex = std::max(U1, 1.0e-6);
        const double thetaI = std::acos(cosThetaI);
        const double fit = 1.0 + thetaI * (-0.876 + thetaI * (0.4265 - 0.0594 * thetaI));
        double b = c - (1.0 + c) * std::pow(1.0 - samplex, fit);
        static const double SQRT_PI_INV = 1.0 / std::sqrt(kPi);
        const double normalization = 1.0 / (1.0 + c + SQRT_PI_INV * tanThetaI * std::exp(-cotThetaI * cotThetaI));
        for (int it = 0; it < 16; it++) {
            if (b < a || c < b) b = 0.5 * (a + c);
            const double xm = refErfinv(b);
            const double value = normalization * (1.0 + b + SQRT_PI_INV * tanThetaI * std::exp(-xm * xm)) - samplex;
            const double derivative = normalization * (1.0 - xm * tanThetaI);
            if (std::abs(value) < 1.0e-6) break;
            if (value > 0.0) c = b;
            else a = b;
            b -= value / derivative;
        }
        *sx = refErfinv(b);
        *sy = refErfinv(2.0 * std::max(U2, 1.0e-6) - 1.0);
    }
    V3 sample(const V3 &wo, P2 u) const {
        const bool flip = wo.z < 0.0;
        const V3 wi = flip ? -wo : wo;
        const V3 ws = normalizeDiv(V3(ax * wi.x, ay * wi.y, wi.z));
        double sx, sy;
        sample11(cosT(ws), u.u0, u.u1, &sx, &sy);
        const double tmp = cosP(ws) * sx - sinP(ws) * sy;
        sy = sinP(ws) * sx + cosP(ws) * sy;
        sx = tmp;
        sx *= ax;
        sy *= ay;
        V3 wh = normalizeDiv(V3(-sx, -sy, 1.0));
        if (flip) wh = -wh;
        return wh;
    }
};

// The BxDFs' hidden generators: `static thread_local Random random` in core/bxdf.cc:18
// (MicrofacetTransmission) and bsdfs/plastic.cc:18 (PlasticBRDF), default seed 0.
inline Sampler &hiddenBxdfRandom() {
    static thread_local Sampler r(0u);
    return r;
}
inline Sampler &hiddenPlasticRandom() {
    static thread_local Sampler r(0u);
    return r;
}
// A hidden draw, for spo_bsdf_sample_uc: with g_ucIn set, the draw is *g_ucIn instead of
// the generator's next number; either way it is recorded in g_ucLast.
thread_local const double *g_ucIn = nullptr;
thread_local double g_ucLast = 0.0;
inline double hiddenDraw(Sampler &r) {
    const double v = g_ucIn ? *g_ucIn : r.get1D();
    g_ucLast = v;
    return v;
}

inline double frDiffuseReflectance(double eta) {   // fresnel.cc:87
    if (eta >= 1.0) return -1.4399 / (eta * eta) + 0.7099 / eta + 0.6681 + 0.0636 * eta;
    return -0.4399f + 0.7099 / eta - 0.3319 / (eta * eta) + 0.0636 / (eta * eta * eta);
}

// One material instantiated at a hit: the single BxDF each of the plugins adds.
struct BSDF {
    int kind = -1;        // SPO_MAT_*, -1 = no component (black Lambert)
    RGB R;                // Lambert reflectance
    GGX ggx{1, 1};
    RGB eta, k;           // conductor
    double ior = 1.0;     // dielectric, rough dielectric, plastic
    bool beckmann = true; // microfacet distribution (rough dielectric, rough conductor)
    Beckmann bk{1, 1};
    RGB Kd, Ks;           // plastic
    double specWeight = 0.0;
    V3 nrm, tan, bin;     // shading frame, bsdf.cc:14-19

    double mD(const V3 &wh) const { return beckmann ? bk.D(wh) : ggx.D(wh); }
    double mG(const V3 &wo, const V3 &wi, const V3 &wh) const { return beckmann ? bk.G(wo, wi, wh) : ggx.G(wo, wi, wh); }
    double mPdf(const V3 &wo, const V3 &wh) const { return beckmann ? bk.pdf(wo, wh) : ggx.pdf(wo, wh); }
    V3 mSample(const V3 &wo, P2 u) const { return beckmann ? bk.sample(wo, u) : ggx.sample(wo, u); }

    // MicrofacetTransmission::f / pdf with a given half vector (bxdf.cc:333, 408)
    RGB mtF(const V3 &wo, const V3 &wi, const V3 &wh) const {
        const double cO = cosT(wo), cI = cosT(wi);
        if (cO == 0.0 || cI == 0.0) return RGB(0.0);
        if (wo.z * dot(wo, wh) <= 0.0) return RGB(0.0);
        if (wi.z * dot(wi, wh) <= 0.0) return RGB(0.0);
        const double F = frDielectric(dot(wo, wh), 1.0, ior);
        if (sameHemi(wo, wi)) return RGB(1.0) * F * mD(wh) * mG(wo, wi, wh) / (4.0 * cO * cI);
        const double eta = dot(wo, wh) > 0.0 ? (ior / 1.0) : (1.0 / ior);
        const double factor = 1.0 / eta;
        const double sd = dot(wo, wh) + eta * dot(wi, wh);
        return RGB(1.0) * (1.0 - F) * std::abs(mD(wh) * mG(wo, wi, wh) * eta * eta * absDot(wi, wh) *
                                            absDot(wo, wh) * factor * factor / (cI * cO * sd * sd));
    }
    double mtPdf(const V3 &wo, const V3 &wi, const V3 &wh) const {
        if (wo.z * dot(wo, wh) <= 0.0) return 0.0;
        if (wi.z * dot(wi, wh) <= 0.0) return 0.0;
        const double F = frDielectric(dot(wo, wh), 1.0, ior);
        if (sameHemi(wo, wi)) return F * mPdf(wo, wh) / (4.0 * absDot(wo, wh));
        const double eta = dot(wo, wh) > 0.0 ? (ior / 1.0) : (1.0 / ior);
        const double sd = dot(wo, wh) + eta * dot(wi, wh);
        const double dwhdwi = std::abs((eta * eta * dot(wi, wh)) / (sd * sd));
        return (1.0 - F) * mPdf(wo, wh) * dwhdwi;
    }
    V3 mtHalf(const V3 &wo, const V3 &wi) const {   // bxdf.cc:321-330 / 396-405
        V3 wh;
        if (sameHemi(wo, wi)) {
            wh = normalizeDiv(wo + wi);
        } else {
            const double eta = cosT(wo) > 0.0 ? (ior / 1.0) : (1.0 / ior);
            wh = normalizeDiv(wo + wi * eta);
        }
        return wh.z >= 0.0 ? wh : -wh;
    }

    int type() const {
        if (kind == SPO_MAT_LAMBERT) return kReflection | kDiffuse;
        if (kind == SPO_MAT_CONDUCTOR) return kReflection | kGlossy;
        if (kind == SPO_MAT_DIELECTRIC) return kReflection | kTransmission | kSpecular;
        if (kind == SPO_MAT_ROUGH_DIELECTRIC) return kReflection | kTransmission | kGlossy;
        if (kind == SPO_MAT_PLASTIC) return kReflection | kSpecular | kDiffuse;
        return 0;
    }
    int numComponents(int t) const { return (kind >= 0 && (type() & t) == type()) ? 1 : 0; }
    V3 toLocal(const V3 &v) const { return {dot(tan, v), dot(bin, v), dot(nrm, v)}; }
    V3 toWorld(const V3 &v) const { return v.x * tan + v.y * bin + v.z * nrm; }

    RGB fLocal(const V3 &wo, const V3 &wi) const {
        if (kind == SPO_MAT_LAMBERT) return R * kInvPi;
        if (kind == SPO_MAT_CONDUCTOR) {   // MicrofacetReflection::f, bxdf.cc:265
            const double cO = std::abs(cosT(wo)), cI = std::abs(cosT(wi));
            V3 wh = wi + wo;
            if (cI == 0.0 || cO == 0.0) return RGB(0.0);
            if (wh.x == 0.0 && wh.y == 0.0 && wh.z == 0.0) return RGB(0.0);
            wh = normalizedMul(wh);
            const RGB F = frConductor(std::abs(dot(wi, wh)), RGB(1.0), eta, k);
            return RGB(1.0) * mD(wh) * mG(wo, wi, wh) * F / (4.0 * cI * cO);
        }
        if (kind == SPO_MAT_DIELECTRIC) {   // FresnelSpecular::f, bxdf.cc:171
            const double F = frDielectric(cosT(wo), 1.0, ior);
            if (sameHemi(wo, wi)) {
                if (dot(V3(-wo.x, -wo.y, wo.z), wi) > 1.0 - 1.0e-4) return RGB(1.0) * F / std::abs(cosT(wi));
            } else {
                const bool entering = cosT(wo) > 0.0;
                const double eI = entering ? 1.0 : ior, eT = entering ? ior : 1.0;
                V3 wt;
                if (!refractV(wo, faceForward(V3(0, 0, 1), wo), eI / eT, &wt)) return RGB(0.0);
                if (dot(wi, wt) > 1.0 - 1.0e-4) return (1.0 - F) * RGB(1.0) / std::abs(cosT(wi));
            }
            return RGB(0.0);
        }
        if (kind == SPO_MAT_ROUGH_DIELECTRIC) {   // MicrofacetTransmission::f, bxdf.cc:315
            if (cosT(wo) == 0.0 || cosT(wi) == 0.0) return RGB(0.0);
            return mtF(wo, wi, mtHalf(wo, wi));
        }
        if (kind == SPO_MAT_PLASTIC) {   // PlasticBRDF::f, plastic.cc:31
            const double Fo = frDielectric(cosT(wo), 1.0, ior);
            if (dot(wi, V3(-wi.x, -wi.y, wi.z)) > 1.0 - kEps) return Fo * Ks / std::abs(cosT(wi));
            const double eta = ior / 1.0, invEta = 1.0 / eta;
            const double Fi = frDielectric(cosT(wi), 1.0, ior);
            const double Fdr = frDiffuseReflectance(eta);
            return (1.0 - Fo) * (1.0 - Fi) * invEta * invEta * Kd * kInvPi / (1.0 - Fdr);
        }
        return RGB(0.0);
    }
    double plasticProbSpecular(const V3 &wo) const {   // plastic.cc:48-50
        const double Fo = frDielectric(cosT(wo), 1.0, ior);
        return (Fo * specWeight) / (Fo * specWeight + (1.0 - Fo) * (1.0 - specWeight));
    }
    double pdfLocal(const V3 &wo, const V3 &wi) const {
        if (kind == SPO_MAT_LAMBERT) return wo.z * wi.z > 0.0 ? std::abs(wi.z) * kInvPi : 0.0;
        if (kind == SPO_MAT_CONDUCTOR) {
            if (!sameHemi(wo, wi)) return 0.0;
            const V3 wh = normalizeDiv(wo + wi);
            return mPdf(wo, wh) / (4.0 * dot(wo, wh));
        }
        if (kind == SPO_MAT_DIELECTRIC) {
            const double F = frDielectric(cosT(wo), 1.0, ior);
            if (sameHemi(wo, wi)) {
                if (dot(V3(-wo.x, -wo.y, wo.z), wi) > 1.0 - 1.0e-4) return F;
            } else {
                const bool entering = cosT(wo) > 0.0;
                const double eI = entering ? 1.0 : ior, eT = entering ? ior : 1.0;
                V3 wt;
                if (!refractV(wo, faceForward(V3(0, 0, 1), wo), eI / eT, &wt)) return 0.0;
                if (dot(wi, wt) > 1.0 - 1.0e-4) return 1.0 - F;
            }
        }
        if (kind == SPO_MAT_ROUGH_DIELECTRIC) return mtPdf(wo, wi, mtHalf(wo, wi));   // bxdf.cc:394
        if (kind == SPO_MAT_PLASTIC) {   // PlasticBRDF::pdf, plastic.cc:71
            const double ps = plasticProbSpecular(wo);
            if (dot(wi, V3(-wi.x, -wi.y, wi.z)) > 1.0 - kEps) return ps;
            return (1.0 - ps) * std::abs(cosT(wi)) * kInvPi;
        }
        return 0.0;
    }

    // BSDF::f, bsdf.cc:49
    RGB f(const V3 &woW, const V3 &wiW, int t) const {
        const V3 wo = toLocal(woW), wi = toLocal(wiW);
        const bool reflect = dot(wiW, nrm) * dot(woW, nrm) > 0.0;
        if (kind < 0 || (type() & t) == 0) return RGB(0.0);
        if ((reflect && (type() & kReflection)) || (!reflect && (type() & kTransmission))) return fLocal(wo, wi);
        return RGB(0.0);
    }
    // BSDF::pdf, bsdf.cc:119
    double pdf(const V3 &woW, const V3 &wiW, int t) const {
        if (kind < 0) return 0.0;
        const V3 wo = toLocal(woW), wi = toLocal(wiW);
        if ((type() & t) == 0) return 0.0;
        return pdfLocal(wo, wi) / 1;
    }
    // BSDF::sample, bsdf.cc:65, with the BxDF samplers of bxdf.cc
    RGB sample(const V3 &woW, V3 *wiW, P2 u, double *pdf, int t, int *sampled) const {
        const int match = numComponents(t);
        if (match == 0) {
            *pdf = 0.0;
            if (sampled) *sampled = 0;
            return RGB(0.0);
        }
        const int comp = std::min(static_cast<int>(u.u0 * match), match - 1);
        const P2 ur{std::min(u.u0 * match - comp, 1.0 - kEps), u.u1};
        const V3 wo = normalizedMul(toLocal(woW));
        if (wo.z == 0.0) return RGB(0.0);
        *pdf = 0.0;
        int st = type();
        V3 wi;
        RGB ret;
        if (kind == SPO_MAT_LAMBERT) {   // BxDF::sample, bxdf.cc:34
            wi = cosineHemisphere(ur);
            if (wo.z < 0.0) wi.z *= -1.0;
            *pdf = pdfLocal(wo, wi);
            ret = fLocal(wo, wi);
        } else if (kind == SPO_MAT_CONDUCTOR) {   // MicrofacetReflection::sample, bxdf.cc:282
            const V3 wh = mSample(wo, ur);
            wi = reflectV(wo, wh);
            if (!sameHemi(wo, wi)) {
                ret = RGB(0.0);
            } else {
                *pdf = mPdf(wo, wh) / (4.0 * dot(wo, wh));
                ret = fLocal(wo, wi);
            }
        } else if (kind == SPO_MAT_ROUGH_DIELECTRIC) {   // MicrofacetTransmission::sample, bxdf.cc:356
            const V3 wh = mSample(wo, ur);
            const double cO = dot(wo, wh.z > 0.0 ? wh : -wh);
            const double F = frDielectric(cO, 1.0, ior);
            bool ok = true;
            if (hiddenDraw(hiddenBxdfRandom()) < F) {
                wi = reflectV(wo, wh);
                if (!sameHemi(wo, wi)) ok = false;
                else st = kReflection | kGlossy;
            } else {
                const double eta = cO > 0.0 ? (1.0 / ior) : (ior / 1.0);
                if (!refractV(wo, wh, eta, &wi) || sameHemi(wo, wi)) ok = false;
                else st = kTransmission | kGlossy;
            }
            if (ok) {
                const V3 whp = wh.z >= 0.0 ? wh : -wh;
                *pdf = mtPdf(wo, wi, whp);
                ret = mtF(wo, wi, whp);
            } else {
                ret = RGB(0.0);
            }
        } else if (kind == SPO_MAT_PLASTIC) {   // PlasticBRDF::sample, plastic.cc:44
            const double Fo = frDielectric(cosT(wo), 1.0, ior);
            const double ps = plasticProbSpecular(wo);
            if (hiddenDraw(hiddenPlasticRandom()) < ps) {
                wi = V3(-wo.x, -wo.y, wo.z);
                *pdf = ps;
                ret = Ks * Fo / std::abs(cosT(wi));
            } else {
                wi = cosineHemisphere(ur);
                const double eta = ior / 1.0, invEta = 1.0 / eta;
                const double Fi = frDielectric(cosT(wi), 1.0, ior);
                const double Fdr = frDiffuseReflectance(eta);
                *pdf = (1.0 - ps) * std::abs(cosT(wi)) * kInvPi;
                ret = (1.0 - Fo) * (1.0 - Fi) * invEta * invEta * Kd * kInvPi / (1.0 - Fdr);
            }
        } else {   // FresnelSpecular::sample, bxdf.cc:198
            const double F = frDielectric(cosT(wo), 1.0, ior);
            if (ur.u0 < F) {
                wi = V3(-wo.x, -wo.y, wo.z);
                st = kSpecular | kReflection;
                *pdf = F;
                ret = RGB(1.0) * (F / std::abs(cosT(wi)));
            } else {
                const bool entering = cosT(wo) > 0.0;
                const double eI = entering ? 1.0 : ior, eT = entering ? ior : 1.0;
                if (!refractV(wo, faceForward(V3(0, 0, 1), wo), eI / eT, &wi)) {
                    ret = RGB(0.0);
                } else {
                    RGB ft = RGB(1.0) * (1.0 - F);
                    ft = ft * ((eI * eI) / (eT * eT));
                    st = kSpecular | kTransmission;
                    *pdf = 1.0 - F;
                    ret = ft / std::abs(cosT(wi));
                }
            }
        }
        if (sampled) *sampled = st;
        if (*pdf == 0.0) {
            if (sampled) *sampled = 0;
            return RGB(0.0);
        }
        *wiW = normalizedMul(toWorld(wi));
        return ret;
    }
};

inline BSDF makeBSDF(const double *m, const V3 &ns, const V3 &ts, const V3 &bs) {
    BSDF b;
    b.nrm = normalizedMul(ns);
    b.tan = normalizedMul(ts);
    b.bin = normalizedMul(bs);
    const int type = static_cast<int>(m[0]);
    if (type == SPO_MAT_LAMBERT) {   // Diffuse::setScatterFuncs, diffuse.cc:23
        b.R = RGB(std::max(0.0, m[1]), std::max(0.0, m[2]), std::max(0.0, m[3]));
        if (!b.R.isBlack()) b.kind = SPO_MAT_LAMBERT;
    } else if (type == SPO_MAT_CONDUCTOR || type == SPO_MAT_CONDUCTOR_BECKMANN) {
        // RoughConductor::setScatterFuncs, roughconductor.cc:38
        b.kind = SPO_MAT_CONDUCTOR;
        const double a = RGB(m[1]).gray();
        b.beckmann = type == SPO_MAT_CONDUCTOR_BECKMANN;
        b.ggx = GGX{a, a};
        b.bk = Beckmann{a, a};
        b.eta = RGB(m[2], m[3], m[4]);
        b.k = RGB(m[5], m[6], m[7]);
    } else if (type == SPO_MAT_ROUGH_DIELECTRIC) {   // RoughDielectric::setScatterFuncs, roughdielectric.cc:41
        const double a = RGB(m[1]).gray();
        b.ior = RGB(m[2]).gray();
        if (a == 0.0) {
            b.kind = SPO_MAT_DIELECTRIC;   // FresnelSpecular when both roughnesses are 0
        } else {
            b.kind = SPO_MAT_ROUGH_DIELECTRIC;
            b.beckmann = m[3] == 0.0;
            b.bk = Beckmann{a, a};
            b.ggx = GGX{a, a};
        }
    } else if (type == SPO_MAT_PLASTIC) {   // Plastic::setScatterFuncs, plastic.cc:112
        b.kind = SPO_MAT_PLASTIC;
        b.Kd = RGB(m[1], m[2], m[3]);
        b.Ks = RGB(m[4], m[5], m[6]);
        b.ior = RGB(m[7]).gray();
        b.specWeight = b.Ks.gray() / (b.Kd.gray() + b.Ks.gray());
    } else {   // Dielectric::setScatterFuncs, dielectric.cc:30
        b.kind = SPO_MAT_DIELECTRIC;
        b.ior = RGB(m[1]).gray();
    }
    return b;
}

inline double powerHeuristic(double f, double g) {   // mis.cc:138
    const double ff = 1 * f, gg = 1 * g;
    return (ff * ff) / (ff * ff + gg * gg);
}

}  // namespace spo

using namespace spo;

struct spo_scene {
    std::vector<Tri> tris;
    std::vector<int32_t> triMat;
    std::vector<double> mats;
    std::vector<RGB> emit;        // per triangle
    std::vector<int> lightTri;    // area light -> triangle (lights vector order)
    std::vector<int> triLight;    // triangle -> light index or -1
    bool hasEnv = false;
    Envmap env;
    BVH bvh;

    int numLights() const { return static_cast<int>(lightTri.size()) + (hasEnv ? 1 : 0); }

    bool intersect(Ray &r, Hit *h) const { return bvh.closest(r, h); }
    bool occluded(const Ray &r) const { return bvh.any(r); }

    RGB areaL(int tri, const V3 &n, const V3 &w) const {   // AreaLight::L, lights/area.cc:29
        return dot(n, w) > 0.0 ? emit[tri] : RGB(0.0);
    }
    // Shape::pdf(Interaction, wi) for a light triangle, core/shape.cc:39
    double triPdf(int tri, const V3 &p, const V3 &n, const V3 &wi) const {
        const Ray ray = spawnRay(p, n, wi);
        double t;
        if (!triHit(tris[tri], ray, &t, nullptr, nullptr)) return 0.0;
        Hit h;
        fillHit(tris[tri], ray, t, &h);
        const V3 d = p - h.pos;
        double ret = dot(d, d) / (absDot(h.n, -wi) * triArea(tris[tri]));
        if (std::isinf(ret)) ret = 0.0;
        return ret;
    }

    // estimateDirectLight, core/mis.cc:35 (surface interaction, no media, specular=false)
    RGB directLight(const Hit &h, const BSDF &b, P2 uShade, int light, P2 uLight) const {
        const int bx = kAll & ~kSpecular;
        RGB Ld(0.0);
        V3 wi;
        double lightPdf = 0.0, bsdfPdf = 0.0;
        const bool isEnv = light >= static_cast<int>(lightTri.size());
        RGB Li(0.0);
        V3 visP;
        V3 visN;
        if (!isEnv) {   // AreaLight::sampleLi + Triangle::sample, area.cc:33, triangle.cc:180
            const int tri = lightTri[light];
            const Tri &T = tris[tri];
            const V3 e1 = T.p[1] - T.p[0], e2 = T.p[2] - T.p[0];
            double u0, u1;
            if (uLight.u0 + uLight.u1 >= 1.0) { u0 = 1.0 - uLight.u0; u1 = 1.0 - uLight.u1; }
            else { u0 = uLight.u0; u1 = uLight.u1; }
            const V3 pos = T.p[0] + u0 * e1 + u1 * e2;
            const V3 nrm = (1.0 - u0 - u1) * T.n + u0 * T.n + u1 * T.n;
            wi = normalizedMul(pos - h.pos);
            lightPdf = triPdf(tri, h.pos, h.n, wi);
            visP = pos;
            visN = nrm;
            Li = areaL(tri, nrm, -wi);
        } else {   // Envmap::sampleLi, envmap.cc:60
            double mapPdf;
            int v;
            const double d1 = env.marg.sample(uLight.u1, &mapPdf, &v);
            double pdf0;
            const double d0 = env.cond[v].sample(uLight.u0, &pdf0, nullptr);
            mapPdf = pdf0 * mapPdf;
            if (mapPdf == 0.0) {
                Li = RGB(0.0);
            } else {
                const double theta = d1 * kPi, phi = d0 * (2.0 * kPi);
                const double ct = std::cos(theta), stt = std::sin(theta);
                const double cp = std::cos(phi), sp = std::sin(phi);
                wi = V3(stt * cp, stt * sp, ct);
                lightPdf = stt == 0.0 ? 0.0 : mapPdf / (2.0 * kPi * kPi * stt);
                visP = h.pos + wi * (2.0 * env.radius);
                visN = V3(0, 0, 0);
                Li = env.mip.lookup(d0, d1);
            }
        }
        if (lightPdf > 0.0 && !Li.isBlack()) {
            const RGB f = b.f(h.wo, wi, bx) * absDot(wi, h.n);
            const double bp = b.pdf(h.wo, wi, bx);
            if (!f.isBlack()) {
                if (occluded(spawnRayTo(h.pos, h.n, visP, visN))) Li = RGB(0.0);
                if (!Li.isBlack()) {
                    const double w = powerHeuristic(lightPdf, bp);
                    Ld = Ld + f * Li * w / lightPdf;
                }
            }
        }
        // BSDF sampling with MIS
        int st = 0;
        RGB f = b.sample(h.wo, &wi, uShade, &bsdfPdf, bx, &st);
        f = f * absDot(wi, h.n);
        const bool spec = (st & kSpecular) != 0;
        if (!f.isBlack() && bsdfPdf > 0.0) {
            double weight = 1.0;
            if (!spec) {
                lightPdf = isEnv ? env.pdfLi(wi) : triPdf(lightTri[light], h.pos, h.n, wi);
                if (lightPdf == 0.0) return Ld;
                weight = powerHeuristic(bsdfPdf, lightPdf);
            }
            Ray ray = spawnRay(h.pos, h.n, wi);
            Hit lh;
            const bool found = intersect(ray, &lh);
            RGB Lr(0.0);
            if (found) {
                if (!isEnv && triLight[lh.prim] == light) Lr = areaL(lh.prim, lh.n, -wi);
            } else if (isEnv) {
                Lr = env.Le(ray.d);
            }
            if (!Lr.isBlack()) Ld = Ld + f * Lr * RGB(1.0) * weight / bsdfPdf;
        }
        return Ld;
    }

    // PathIntegrator::Li, integrators/path/path.cc:42
    RGB Li(Ray ray, Sampler &sampler, int maxDepth) const {
        RGB L(0.0), beta(1.0);
        bool specularBounce = false;
        const int nL = numLights();
        for (int bounces = 0;; bounces++) {
            Hit h;
            const bool hit = intersect(ray, &h);
            if (bounces == 0 || specularBounce) {
                if (hit) {
                    if (triLight[h.prim] >= 0) L = L + beta * areaL(h.prim, h.n, -ray.d);
                } else if (hasEnv) {
                    L = L + beta * env.Le(ray.d);
                }
            }
            if (!hit || bounces >= maxDepth) break;
            const V3 &ns = h.n;
            const BSDF b = makeBSDF(&mats[SPO_MAT_STRIDE * triMat[h.prim]], ns, h.dpdu, h.dpdv);
            if (b.numComponents(kAll & ~kSpecular) > 0 && nL > 0) {   // uniformSampleOneLight, mis.cc:21
                const int light = std::min(static_cast<int>(sampler.get1D() * nL), nL - 1);
                const P2 uLight = sampler.get2D();
                const P2 uShade = sampler.get2D();
                L = L + beta * (nL * directLight(h, b, uShade, light, uLight));
            }
            V3 wi;
            double pdf = 0.0;
            int st = 0;
            const RGB ref = b.sample(-ray.d, &wi, sampler.get2D(), &pdf, kAll, &st);
            if (ref.isBlack() || pdf == 0.0) break;
            beta = beta * (ref * absDot(wi, ns) / pdf);
            specularBounce = (st & kSpecular) != 0;
            ray = spawnRay(h.pos, h.n, wi);
            if (bounces > 3) {
                const double q = std::min(0.95, beta.gray());
                if (sampler.get1D() > q) break;
                beta = beta / q;
            }
        }
        return L;
    }

    // DirectLightingIntegrator::Li, integrators/directlighting/directlighting.cc:21.
    // Its specular recursion (core/integrator.cc:112-152) samples BxDFs of type
    // Reflection|Specular or Transmission|Specular alone (bsdf.cc:28 matching); none
    // of the three materials has one, so it never recurses.
    RGB LiDirect(Ray ray, Sampler &sampler, int maxDepth) const {
        Hit h;
        if (!intersect(ray, &h)) return hasEnv ? env.Le(ray.d) : RGB(0.0);   // sum of Light::Le(ray)
        RGB L(0.0);
        if (triLight[h.prim] >= 0) L = areaL(h.prim, h.n, -ray.d);        // depth 0: isect.Le(-dir)
        const int nL = numLights();
        if (nL > 0) {   // uniformSampleOneLight, core/mis.cc:21
            const BSDF b = makeBSDF(&mats[SPO_MAT_STRIDE * triMat[h.prim]], h.n, h.dpdu, h.dpdv);
            const int light = std::min(static_cast<int>(sampler.get1D() * nL), nL - 1);
            const P2 uLight = sampler.get2D();
            const P2 uShade = sampler.get2D();
            // unconditional, unlike the path integrator's guard (path.cc:77): BSDF::f matches
            // a BxDF sharing any type bit, so plastic's diffuse lobe is light-sampled here
            if (b.kind >= 0) L = L + nL * directLight(h, b, uShade, light, uLight);
        }
        if (1 < maxDepth) {
            // specularReflect / specularTransmit draw their 2D sample before finding no
            // matching BxDF (core/integrator.cc:120,142)
            (void)sampler.get2D();
            (void)sampler.get2D();
        }
        return L;
    }
};

namespace {
template <class F>
void parallelRange(int64_t n, int nthreads, int64_t chunk, F &&body) {
    if (nthreads <= 1) {
        // one fresh thread, whose hidden BxDF generators start from their seed (as a
        // fresh reference thread's do)
        std::thread th([&]() {
            for (int64_t i = 0; i < n; i += chunk) body(i, std::min(n, i + chunk));
        });
        th.join();
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++) {
        pool.emplace_back([&]() {
            for (;;) {
                const int64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                body(b, std::min(n, b + chunk));
            }
        });
    }
    for (auto &th : pool) th.join();
}
}  // namespace

extern "C" {

const char *spo_name(void) { return "port"; }

spo_scene *spo_scene_create(int ntri, const double *verts, const int32_t *tri_mat, int nmat,
                            const double *mats, const double *tri_emit, int env_w, int env_h,
                            const float *env, int /*use_simd*/) {
    auto *s = new spo_scene();
    s->tris.resize(ntri);
    s->triMat.assign(tri_mat, tri_mat + ntri);
    s->mats.assign(mats, mats + static_cast<size_t>(nmat) * SPO_MAT_STRIDE);
    s->emit.assign(ntri, RGB(0.0));
    s->triLight.assign(ntri, -1);
    Box bounds;
    for (int i = 0; i < ntri; i++) {
        Tri &T = s->tris[i];
        for (int k = 0; k < 3; k++) {
            T.p[k] = V3(verts[9 * i + 3 * k], verts[9 * i + 3 * k + 1], verts[9 * i + 3 * k + 2]);
            bounds.merge(T.p[k]);
        }
        T.n = normalizedMul(cross(T.p[1] - T.p[0], T.p[2] - T.p[0]));
        if (tri_emit) {
            const double *e = tri_emit + 3 * i;
            if (e[0] != 0.0 || e[1] != 0.0 || e[2] != 0.0) {
                s->emit[i] = RGB(e[0], e[1], e[2]);
                s->triLight[i] = static_cast<int>(s->lightTri.size());
                s->lightTri.push_back(i);
            }
        }
    }
    if (env) {
        Image img;
        img.w = env_w;
        img.h = env_h;
        img.px.resize(static_cast<size_t>(env_w) * env_h);
        for (size_t i = 0; i < img.px.size(); i++) img.px[i] = RGB(env[3 * i], env[3 * i + 1], env[3 * i + 2]);
        s->hasEnv = true;
        s->env.init(img, 0.5 * (bounds.lo + bounds.hi), 0.5 * norm(bounds.hi - bounds.lo));
    }
    s->bvh.build(s->tris);
    return s;
}

double spo_triangle_area(const double *v) {
    Tri T;
    for (int k = 0; k < 3; k++) T.p[k] = V3(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
    return triArea(T);
}

int spo_box_intersect(const double *lo, const double *hi, const double *org, const double *dir, double tmax,
                      double *tnear, double *tfar) {
    Box b;
    b.lo = V3(lo[0], lo[1], lo[2]);
    b.hi = V3(hi[0], hi[1], hi[2]);
    return b.hit(Ray(V3(org[0], org[1], org[2]), V3(dir[0], dir[1], dir[2]), tmax), tnear, tfar) ? 1 : 0;
}

void spo_ray_invdir(const double *org, const double *dir, double *inv) {
    const Ray r(V3(org[0], org[1], org[2]), V3(dir[0], dir[1], dir[2]));
    inv[0] = r.inv.x;
    inv[1] = r.inv.y;
    inv[2] = r.inv.z;
}

void spo_scene_destroy(spo_scene *s) { delete s; }

int spo_scene_num_lights(const spo_scene *s) { return s->numLights(); }

int spo_trace(spo_scene *s, int any, int64_t n, const double *org, const double *dir,
              const double *tmax, int32_t *prim, double *t, uint8_t *hit, int nthreads) {
    parallelRange(n, nthreads, 256, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray ray(V3(org[3 * i], org[3 * i + 1], org[3 * i + 2]), V3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]),
                    tmax ? tmax[i] : kInf);
            if (any) {
                const bool h = s->occluded(ray);
                if (hit) hit[i] = h ? 1 : 0;
            } else {
                Hit hh;
                const bool h = s->intersect(ray, &hh);
                if (prim) prim[i] = h ? hh.prim : -1;
                if (t) t[i] = h ? ray.maxDist : 0.0;
                if (hit) hit[i] = h ? 1 : 0;
            }
        }
    });
    return 0;
}

}  // extern "C"

namespace {
// Film window render shared by the integrators: radiance(scene, ray, sampler) gives Li.
template <class F>
int renderWindow(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h, int spp,
                 uint32_t seed, double *sum, double *sumsq, int nthreads, F radiance) {
    const Camera camera(cam, W, H);
    const int64_t npix = static_cast<int64_t>(w) * h;
    parallelRange(npix, nthreads, 1, [&](int64_t b, int64_t e) {
        for (int64_t q = b; q < e; q++) {
            const int fy = fy0 + static_cast<int>(q / w);
            const int fx = fx0 + static_cast<int>(q % w);
            const int x = W - 1 - fx, y = fy;   // film pixel (W-1-x, y), integrator.cc:88
            Sampler sampler(spo_pixel_seed(seed, static_cast<uint32_t>(fy * W + fx)));
            double acc[3] = {0, 0, 0}, acc2[3] = {0, 0, 0};
            for (int k = 0; k < spp; k++) {
                const P2 film = sampler.get2D();
                (void)sampler.get2D();   // lens sample (pinhole camera ignores it)
                V3 o, d;
                camera.spawnRay(x, y, film, &o, &d);
                const RGB L = radiance(Ray(o, d), sampler);
                const double c[3] = {L.r, L.g, L.b};
                for (int j = 0; j < 3; j++) {
                    acc[j] += c[j];
                    acc2[j] += c[j] * c[j];
                }
            }
            for (int j = 0; j < 3; j++) {
                sum[3 * q + j] = acc[j];
                sumsq[3 * q + j] = acc2[j];
            }
        }
    });
    return 0;
}
}  // namespace

extern "C" {
int spo_render(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h, int spp,
               int max_depth, uint32_t seed, double *sum, double *sumsq, int nthreads) {
    return renderWindow(s, cam, W, H, fx0, fy0, w, h, spp, seed, sum, sumsq, nthreads,
                        [&](const Ray &r, Sampler &smp) { return s->Li(r, smp, max_depth); });
}

int spo_render_direct(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h, int spp,
                      int max_depth, uint32_t seed, double *sum, double *sumsq, int nthreads) {
    return renderWindow(s, cam, W, H, fx0, fy0, w, h, spp, seed, sum, sumsq, nthreads,
                        [&](const Ray &r, Sampler &smp) { return s->LiDirect(r, smp, max_depth); });
}

int spo_bsdf_eval(const double *mat, int64_t n, const double *wo, const double *wi, double *f, double *pdf) {
    V3 ts, bs;
    coordSystem(V3(0, 0, 1), &ts, &bs);
    const BSDF b = makeBSDF(mat, normalizeDiv(cross(V3(1, 0, 0), V3(0, 1, 0))), V3(1, 0, 0), V3(0, 1, 0));
    for (int64_t i = 0; i < n; i++) {
        const V3 o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), d(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        const RGB v = b.f(o, d, kAll);
        f[3 * i] = v.r;
        f[3 * i + 1] = v.g;
        f[3 * i + 2] = v.b;
        pdf[i] = b.pdf(o, d, kAll);
    }
    return 0;
}

int spo_bsdf_sample(const double *mat, int64_t n, const double *wo, const double *u, double *wi, double *f,
                    double *pdf, int32_t *type) {
    const BSDF b = makeBSDF(mat, normalizeDiv(cross(V3(1, 0, 0), V3(0, 1, 0))), V3(1, 0, 0), V3(0, 1, 0));
    // in a fresh thread: the hidden BxDF generators start from their seed
    std::thread th([&]() {
        for (int64_t i = 0; i < n; i++) {
            const V3 o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
            V3 d(0, 0, 0);
            double p = 0.0;
            int st = 0;
            const RGB v = b.sample(o, &d, P2{u[2 * i], u[2 * i + 1]}, &p, kAll, &st);
            wi[3 * i] = d.x;
            wi[3 * i + 1] = d.y;
            wi[3 * i + 2] = d.z;
            f[3 * i] = v.r;
            f[3 * i + 1] = v.g;
            f[3 * i + 2] = v.b;
            pdf[i] = p;
            type[i] = st;
        }
    });
    th.join();
    return 0;
}

// spo_bsdf_sample with the hidden draws made visible: ucIn == NULL draws them from the
// hidden generators (fresh thread, as spo_bsdf_sample) and reports each row's draw in
// ucOut (NaN for a row that took none); otherwise row i's draw is ucIn[i].
int spo_bsdf_sample_uc(const double *mat, int64_t n, const double *wo, const double *u, const double *ucIn,
                       double *wi, double *f, double *pdf, int32_t *type, double *ucOut) {
    const BSDF b = makeBSDF(mat, normalizeDiv(cross(V3(1, 0, 0), V3(0, 1, 0))), V3(1, 0, 0), V3(0, 1, 0));
    std::thread th([&]() {
        for (int64_t i = 0; i < n; i++) {
            const V3 o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
            V3 d(0, 0, 0);
            double p = 0.0;
            int st = 0;
            g_ucIn = ucIn ? ucIn + i : nullptr;
            g_ucLast = std::numeric_limits<double>::quiet_NaN();
            const RGB v = b.sample(o, &d, P2{u[2 * i], u[2 * i + 1]}, &p, kAll, &st);
            g_ucIn = nullptr;
            if (ucOut) ucOut[i] = g_ucLast;
            wi[3 * i] = d.x;
            wi[3 * i + 1] = d.y;
            wi[3 * i + 2] = d.z;
            f[3 * i] = v.r;
            f[3 * i + 1] = v.g;
            f[3 * i + 2] = v.b;
            pdf[i] = p;
            type[i] = st;
        }
    });
    th.join();
    return 0;
}

}  // extern "C"
