// ORACLE -- test infrastructure only.  CPU restatement of the PLTFalcor PLT math used as the
// parity checker for the CUDA kernels; never linked into the product library.
//
// Small vector / matrix / complex helpers with Slang semantics: float2x2(a,b,c,d) is row-major
// [[a,b],[c,d]], mul(M, v) is M*v, dot products sum left to right.
// Follows Source/Falcor/Utils/Math/MathHelpers.slang (complex ops :822-837, tryInvert :484-498,
// ident2/4 :571-582, perp_stark :609-623, sinc :840-843, factorial :813-818, BesselJ :851-885,
// truncated Box-Muller :416-450) and Utils/Math/MathConstants.slangh.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace plt_oracle {

// ---------------------------------------------------------------------------------------------
// Operation counting: a Real type that counts FP32 pipe ops and special-function ops.  Used to
// derive the algorithmic work per query for the roofline (FMA-class ops and SFU-class ops).
// ---------------------------------------------------------------------------------------------
struct OpCounts { uint64_t fp = 0, sfu = 0, div = 0, cmp = 0; };
inline OpCounts& op_counts() { static thread_local OpCounts c; return c; }

struct CF {
    double v;
    CF() : v(0) {}
    CF(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
    explicit operator int() const { return (int)v; }
    explicit operator unsigned() const { return (unsigned)v; }
};
// Products and sums with an exact zero operand are the structural zeros of the sparse Mueller /
// rotation matrices; they are not counted as algorithmic work.
inline CF operator+(CF a, CF b) { if (a.v != 0.0 && b.v != 0.0) op_counts().fp++; return CF(a.v + b.v); }
inline CF operator-(CF a, CF b) { if (a.v != 0.0 && b.v != 0.0) op_counts().fp++; return CF(a.v - b.v); }
inline CF operator*(CF a, CF b) { if (a.v != 0.0 && b.v != 0.0) op_counts().fp++; return CF(a.v * b.v); }
inline CF operator/(CF a, CF b) { op_counts().div++; return CF(a.v / b.v); }
inline CF operator-(CF a) { return CF(-a.v); }
inline CF& operator+=(CF& a, CF b) { a = a + b; return a; }
inline CF& operator-=(CF& a, CF b) { a = a - b; return a; }
inline CF& operator*=(CF& a, CF b) { a = a * b; return a; }
inline CF& operator/=(CF& a, CF b) { a = a / b; return a; }
inline bool operator<(CF a, CF b) { op_counts().cmp++; return a.v < b.v; }
inline bool operator>(CF a, CF b) { op_counts().cmp++; return a.v > b.v; }
inline bool operator<=(CF a, CF b) { op_counts().cmp++; return a.v <= b.v; }
inline bool operator>=(CF a, CF b) { op_counts().cmp++; return a.v >= b.v; }
inline bool operator==(CF a, CF b) { op_counts().cmp++; return a.v == b.v; }
inline bool operator!=(CF a, CF b) { op_counts().cmp++; return a.v != b.v; }

// ---------------------------------------------------------------------------------------------
// Monte Carlo arithmetic (random rounding): a binary32 type whose every operation computes the
// result in double and rounds it to one of the two neighbouring floats at random.  The spread of
// results between runs with different seeds measures how sensitive a query is to FP32 rounding,
// which bounds how closely two FP32 implementations can agree (tests use it as the conditioning
// allowance).
// ---------------------------------------------------------------------------------------------
inline uint64_t& sr_state() { static thread_local uint64_t s = 0x9E3779B97F4A7C15ull; return s; }
inline void sr_seed(uint64_t seed, uint64_t index) { sr_state() = (seed * 0x9E3779B97F4A7C15ull) ^ (index * 0xBF58476D1CE4E5B9ull) ^ 0x94D049BB133111EBull; }
inline float sr_round(double x) {
    const float f = (float)x;
    if (!std::isfinite(x) || (double)f == x) return f;
    uint64_t& s = sr_state();
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    const float up = (double)f > x ? f : std::nextafter(f, INFINITY);
    const float down = (double)f < x ? f : std::nextafter(f, -INFINITY);
    return (s >> 32) & 1u ? up : down;
}
struct SR {
    float v;
    SR() : v(0) {}
    SR(double x) : v((float)x) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return v; }
    explicit operator int() const { return (int)v; }
    explicit operator unsigned() const { return (unsigned)v; }
};
inline SR sr(double x) { SR r; r.v = sr_round(x); return r; }
inline SR operator+(SR a, SR b) { return sr((double)a.v + (double)b.v); }
inline SR operator-(SR a, SR b) { return sr((double)a.v - (double)b.v); }
inline SR operator*(SR a, SR b) { return sr((double)a.v * (double)b.v); }
inline SR operator/(SR a, SR b) { return sr((double)a.v / (double)b.v); }
inline SR operator-(SR a) { SR r; r.v = -a.v; return r; }
inline SR& operator+=(SR& a, SR b) { a = a + b; return a; }
inline SR& operator-=(SR& a, SR b) { a = a - b; return a; }
inline SR& operator*=(SR& a, SR b) { a = a * b; return a; }
inline SR& operator/=(SR& a, SR b) { a = a / b; return a; }
inline bool operator<(SR a, SR b) { return a.v < b.v; }
inline bool operator>(SR a, SR b) { return a.v > b.v; }
inline bool operator<=(SR a, SR b) { return a.v <= b.v; }
inline bool operator>=(SR a, SR b) { return a.v >= b.v; }
inline bool operator==(SR a, SR b) { return a.v == b.v; }
inline bool operator!=(SR a, SR b) { return a.v != b.v; }

// Scalar math shims.  For CF each special function counts as one SFU-class op (sqrt, rsqrt,
// exp, log, sin, cos, pow = exp+log, atan2/acos = polynomial sequences, counted as 4 FP + 1 SFU).
#define PLT_ORACLE_UNARY(NAME, STD, SFU, FP)                                                    \
    inline float NAME(float x) { return std::STD(x); }                                          \
    inline double NAME(double x) { return std::STD(x); }                                        \
    inline CF NAME(CF x) { op_counts().sfu += SFU; op_counts().fp += FP; return CF(std::STD(x.v)); } \
    inline SR NAME(SR x) { return sr(std::STD((double)x.v)); }
PLT_ORACLE_UNARY(o_sqrt, sqrt, 1, 0)
PLT_ORACLE_UNARY(o_exp, exp, 1, 1)
PLT_ORACLE_UNARY(o_log, log, 1, 1)
PLT_ORACLE_UNARY(o_sin, sin, 1, 2)
PLT_ORACLE_UNARY(o_cos, cos, 1, 2)
PLT_ORACLE_UNARY(o_acos, acos, 1, 8)
PLT_ORACLE_UNARY(o_floor, floor, 0, 1)
PLT_ORACLE_UNARY(o_ceil, ceil, 0, 1)
#undef PLT_ORACLE_UNARY
inline float o_abs(float x) { return std::fabs(x); }
inline double o_abs(double x) { return std::fabs(x); }
inline CF o_abs(CF x) { return CF(std::fabs(x.v)); }
inline SR o_abs(SR x) { SR r; r.v = std::fabs(x.v); return r; }
inline SR o_pow(SR x, SR y) { return sr(std::pow((double)x.v, (double)y.v)); }
inline SR o_atan2(SR y, SR x) { return sr(std::atan2((double)y.v, (double)x.v)); }
inline bool o_isfinite(SR x) { return std::isfinite(x.v); }
inline float o_fval(SR x) { return x.v; }
inline float o_pow(float x, float y) { return std::pow(x, y); }
inline double o_pow(double x, double y) { return std::pow(x, y); }
inline CF o_pow(CF x, CF y) { op_counts().sfu += 2; op_counts().fp += 2; return CF(std::pow(x.v, y.v)); }
inline float o_atan2(float y, float x) { return std::atan2(y, x); }
inline double o_atan2(double y, double x) { return std::atan2(y, x); }
inline CF o_atan2(CF y, CF x) { op_counts().sfu += 1; op_counts().fp += 12; return CF(std::atan2(y.v, x.v)); }
inline bool o_isfinite(float x) { return std::isfinite(x); }
inline bool o_isfinite(double x) { return std::isfinite(x); }
inline bool o_isfinite(CF x) { return std::isfinite(x.v); }
inline float o_fval(float x) { return x; }
inline float o_fval(double x) { return (float)x; }
inline float o_fval(CF x) { return (float)x.v; }

template <class R> inline R o_min(R a, R b) { return (b < a) ? b : a; }
template <class R> inline R o_max(R a, R b) { return (a < b) ? b : a; }
template <class R> inline R o_clamp(R x, R lo, R hi) { return o_min(o_max(x, lo), hi); }
template <class R> inline R sqr(R x) { return x * x; }
// HLSL sign(): -1, 0 or +1
template <class R> inline R o_sign(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
template <class R> inline R lerp(R a, R b, R t) { return a + (b - a) * t; }

// Constants (MathConstants.slangh).  Slang folds them as float literals; in the FP64 build they
// are the double values.
constexpr double K_PI = 3.14159265358979323846;
constexpr double K_2PI = 6.28318530717958647693;
constexpr double K_4PI = 12.5663706143591729539;
constexpr double K_1_PI = 0.318309886183790671538;
constexpr double K_1_2PI = 0.159154943091895335769;
constexpr float K_FLT_EPSILON = 1.192092896e-07F;

// ---------------------------------------------------------------------------------------------
template <class R> struct V2 { R x, y; };
template <class R> struct V3 { R x, y, z; };
template <class R> struct V4 { R x, y, z, w; };

template <class R> inline V2<R> v2(R x, R y) { return {x, y}; }
template <class R> inline V3<R> v3(R x, R y, R z) { return {x, y, z}; }

template <class R> inline V2<R> operator+(V2<R> a, V2<R> b) { return {a.x + b.x, a.y + b.y}; }
template <class R> inline V2<R> operator-(V2<R> a, V2<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> inline V2<R> operator*(V2<R> a, R s) { return {a.x * s, a.y * s}; }
template <class R> inline V2<R> operator/(V2<R> a, R s) { return {a.x / s, a.y / s}; }
template <class R> inline V2<R> operator-(V2<R> a) { return {-a.x, -a.y}; }
template <class R> inline R dot(V2<R> a, V2<R> b) { return a.x * b.x + a.y * b.y; }

template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length(V3<R> a) { return o_sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) { return a / length(a); }

template <class R> inline V4<R> operator+(V4<R> a, V4<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class R> inline V4<R> operator*(V4<R> a, R s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class R> inline V4<R> operator*(R s, V4<R> a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }

// 2x2 matrix, row-major m[row][col]
template <class R> struct M2 { R m[2][2]; };
template <class R> inline M2<R> m2(R a, R b, R c, R d) { M2<R> r; r.m[0][0] = a; r.m[0][1] = b; r.m[1][0] = c; r.m[1][1] = d; return r; }
template <class R> inline M2<R> ident2(R d = R(1)) { return m2(d, R(0), R(0), d); }
template <class R> inline M2<R> transpose(M2<R> a) { return m2(a.m[0][0], a.m[1][0], a.m[0][1], a.m[1][1]); }
template <class R> inline R determinant(M2<R> a) { return a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]; }
template <class R> inline M2<R> operator*(M2<R> a, R s) { return m2(a.m[0][0] * s, a.m[0][1] * s, a.m[1][0] * s, a.m[1][1] * s); }
template <class R> inline M2<R> operator*(R s, M2<R> a) { return m2(s * a.m[0][0], s * a.m[0][1], s * a.m[1][0], s * a.m[1][1]); }
template <class R> inline M2<R> operator/(M2<R> a, R s) { return m2(a.m[0][0] / s, a.m[0][1] / s, a.m[1][0] / s, a.m[1][1] / s); }
template <class R> inline M2<R> operator+(M2<R> a, M2<R> b) { return m2(a.m[0][0] + b.m[0][0], a.m[0][1] + b.m[0][1], a.m[1][0] + b.m[1][0], a.m[1][1] + b.m[1][1]); }
template <class R> inline M2<R> operator-(M2<R> a, M2<R> b) { return m2(a.m[0][0] - b.m[0][0], a.m[0][1] - b.m[0][1], a.m[1][0] - b.m[1][0], a.m[1][1] - b.m[1][1]); }
template <class R> inline V2<R> mul(M2<R> a, V2<R> v) { return {a.m[0][0] * v.x + a.m[0][1] * v.y, a.m[1][0] * v.x + a.m[1][1] * v.y}; }
template <class R> inline M2<R> mul(M2<R> a, M2<R> b) {
    M2<R> r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j];
    return r;
}

// 4x4 matrix, row-major
template <class R> struct M4 { R m[4][4]; };
template <class R> inline M4<R> zero4() { M4<R> r; for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) r.m[i][j] = R(0); return r; }
template <class R> inline V4<R> mul(const M4<R>& a, V4<R> v) {
    return {a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z + a.m[0][3] * v.w,
            a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z + a.m[1][3] * v.w,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z + a.m[2][3] * v.w,
            a.m[3][0] * v.x + a.m[3][1] * v.y + a.m[3][2] * v.z + a.m[3][3] * v.w};
}
template <class R> inline M4<R> mul(const M4<R>& a, const M4<R>& b) {
    M4<R> r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return r;
}
template <class R> inline M4<R> operator+(const M4<R>& a, const M4<R>& b) {
    M4<R> r;
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}
template <class R> inline M4<R> operator*(R s, const M4<R>& a) {
    M4<R> r;
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) r.m[i][j] = s * a.m[i][j];
    return r;
}

// ---- complex numbers as float2 (MathHelpers.slang:822-837) ----
template <class R> inline V2<R> c_t(R re, R im = R(0)) { return {re, im}; }
template <class R> inline R cnorm2(V2<R> z) { return dot(z, z); }
template <class R> inline R cabs(V2<R> z) { return o_sqrt(cnorm2(z)); }
template <class R> inline V2<R> csqrt(V2<R> z) {
    const R r = cabs(z);
    const R a = o_sqrt(o_max(R(0), r + z.x) / R(2));
    const R b = o_sqrt(o_max(R(0), r - z.x) / R(2));
    return c_t(a, o_sign(z.y) * b);
}
template <class R> inline V2<R> cconj(V2<R> z) { return c_t(z.x, -z.y); }
template <class R> inline V2<R> cmul(V2<R> a, V2<R> b) { return c_t(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <class R> inline V2<R> cdiv(V2<R> a, V2<R> b) { return cmul(a, cconj(b)) / cnorm2(b); }
template <class R> inline V2<R> csqr(V2<R> z) { return cmul(z, z); }
template <class R> inline R carg(V2<R> z) { return o_atan2(z.y, z.x); }

// tryInvert 2x2, MathHelpers.slang:484-498 (threshold compared in double, as written)
template <class R> inline bool tryInvert(M2<R> a, M2<R>& inv) {
    const R det = determinant(a);
    if (o_abs(det) < R(4e-6)) return false;
    const R invdet = R(1) / det;
    inv.m[0][0] = a.m[1][1] * invdet;
    inv.m[1][1] = a.m[0][0] * invdet;
    inv.m[0][1] = -a.m[0][1] * invdet;
    inv.m[1][0] = -a.m[1][0] * invdet;
    return true;
}

// perp_stark, MathHelpers.slang:609-623
template <class R> inline V3<R> perp_stark(V3<R> u) {
    const V3<R> a = {o_abs(u.x), o_abs(u.y), o_abs(u.z)};
    const unsigned uyx = (a.x - a.y) < R(0) ? 1u : 0u;
    const unsigned uzx = (a.x - a.z) < R(0) ? 1u : 0u;
    const unsigned uzy = (a.y - a.z) < R(0) ? 1u : 0u;
    const unsigned xm = uyx & uzx;
    const unsigned ym = (1u ^ xm) & uzy;
    const unsigned zm = 1u ^ (xm | ym);
    return normalize(cross(u, V3<R>{R((double)xm), R((double)ym), R((double)zm)}));
}

// factorial table and BesselJ approximation, MathHelpers.slang:813-885
inline unsigned factorial(unsigned n) {
    static const unsigned table[13] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880, 3628800, 39916800, 479001600};
    return n < 13 ? table[n] : 0u;
}
template <class R> inline R BesselJ_saa(int nu, R x) {
    if (nu >= 7) return R(std::nan(""));
    const R x2 = sqr(x);
    const R x4 = sqr(x2);
    const R x6 = x2 * x4;
    const R x8 = sqr(x4);
    const R s = R(6) * o_pow(x / R(2), R((double)nu));
    const R a = R(1) / (R(6) * R((double)factorial((unsigned)nu)));
    const R b = -x2 / (R(24) * R((double)factorial((unsigned)nu + 1)));
    const R c1 = R(11) * x8 - R(864) * R((double)(6 + nu)) *
                 (x6 - R(12) * (R(5) + R((double)nu)) *
                           (R(3) * x4 + R(32) * R((double)(4 + nu)) * (R(-2) * x2 + R(27) * R((double)(3 + nu)))));
    const R c = c1 / R((double)factorial((unsigned)(6 + nu))) * x4 * R(5.652695401144601e-10);
    return s * (a + b + c);
}
template <class R> inline R BesselJ_laa(int nu, R x) {
    return o_sqrt(R(2) / R(K_PI) / x) * o_cos(x - R((double)nu) * R(K_PI) / R(2) - R(K_PI) / R(4));
}
template <class R> inline R BesselJ(int nu, R x) {
    const R t = (nu > 0 || (-nu) % 2 == 0) ? R(1) : R(-1);
    nu = nu < 0 ? -nu : nu;
    const R cutoff = R((double)nu) + R(1);
    const R interp = cutoff / R(10);
    const R laa = BesselJ_laa(nu, x);
    const R saa = BesselJ_saa(nu, x);
    return (nu >= 7 || o_abs(x) >= cutoff + interp)
               ? laa * t
               : lerp(saa, laa, o_max(R(0), o_min(R(1), R(0.5) * (x - cutoff - interp) / interp))) * t;
}

template <class R> inline R sinc(R x) { return o_sin(x) / x; }

// sample_boxmueller_truncated / boxmueller_truncated_pdf, MathHelpers.slang:416-450
template <class R> inline V2<R> sample_boxmueller_truncated(V2<R> u, V2<R> mean, R sigma2, R& pdf) {
    const R l = o_sqrt(o_min(R(1), dot(mean, mean)));
    const R coso = o_sqrt(o_max(R(0), R(1) - dot(mean, mean)));
    const R phi_i = (mean.x != R(0) || mean.y != R(0)) ? o_atan2(mean.y, mean.x) : R(0);
    const R s = o_exp(R(-0.5) * sqr(R(1) + l) / sigma2);
    const R x = (R(1) - s) * o_max(R(K_FLT_EPSILON), u.x) + s;
    const R r = o_sqrt(R(-2) * sigma2 * o_log(x));
    const R max_phi = (r < R(K_FLT_EPSILON) || l < R(K_FLT_EPSILON))
                          ? R(K_PI)
                          : o_acos(o_clamp((sqr(r) + sqr(l) - R(1)) / (R(2) * r * l), R(-1), R(1)));
    const R phi = phi_i + R(K_PI) + max_phi * (R(2) * u.y - R(1));
    const V2<R> p = {r * o_cos(phi), r * o_sin(phi)};
    pdf = R(0.5) * x / (max_phi * sigma2) * coso;
    return p + mean;
}
template <class R> inline R boxmueller_truncated_pdf(V2<R> wo, V2<R> mean, R sigma2) {
    const R l = o_sqrt(o_min(R(1), dot(mean, mean)));
    const R coso = o_sqrt(o_max(R(0), R(1) - dot(mean, mean)));
    wo = wo - mean;
    const R r2 = dot(wo, wo);
    const R x = o_exp(R(-0.5) * r2 / sigma2);
    const R r = o_sqrt(r2);
    const R max_phi = (r < R(K_FLT_EPSILON) || l < R(K_FLT_EPSILON))
                          ? R(K_PI)
                          : o_acos(o_clamp((sqr(r) + sqr(l) - R(1)) / (R(2) * r * l), R(-1), R(1)));
    return R(0.5) * x / (max_phi * sigma2) * coso;
}

// Concentric cosine-hemisphere sampling (MathHelpers.slang:305-338)
template <class R> inline V2<R> sample_disk_concentric(V2<R> u) {
    u = v2(R(2) * u.x - R(1), R(2) * u.y - R(1));
    if (u.x == R(0) && u.y == R(0)) return u;
    R phi, r;
    if (o_abs(u.x) > o_abs(u.y)) {
        r = u.x;
        phi = (u.y / u.x) * R(K_PI / 4.0);
    } else {
        r = u.y;
        phi = R(K_PI / 2.0) - (u.x / u.y) * R(K_PI / 4.0);
    }
    return v2(r * o_cos(phi), r * o_sin(phi));
}
template <class R> inline V3<R> sample_cosine_hemisphere_concentric(V2<R> u, R& pdf) {
    const V2<R> d = sample_disk_concentric(u);
    const R z = o_sqrt(o_max(R(0), R(1) - dot(d, d)));
    pdf = z * R(K_1_PI);
    return {d.x, d.y, z};
}
template <class R> inline R cosine_hemisphere_concentric_pdf(V3<R> wo) { return wo.z * R(K_1_PI); }

}  // namespace plt_oracle
