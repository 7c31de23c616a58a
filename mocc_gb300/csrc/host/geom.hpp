// Planar geometry primitives used by the modular ray tracer.
//
// The arithmetic follows MOCC's geometry kernel so that traced segment
// lengths agree with MOCC's own known-answer tests to ~1e-15:
//   fuzzy comparisons      src/util/fp_utils.hpp:39-120
//   Point2 / Midpoint      src/core/geometry/points.hpp
//   line/circle crossings  src/core/geometry/geom.hpp (Intersect)
//   Box::intersect         src/core/geometry/box.cpp
//   Direction / Angle      src/core/geometry/direction.hpp:57-188, angle.cpp
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <stdexcept>
#include <string>

namespace mocgpu {

constexpr double kPi = 3.1415926535897932;
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kHalfPi = 0.5 * kPi;
constexpr double kFourPi = 4.0 * kPi;
constexpr double kFuzz = 200 * std::numeric_limits<double>::epsilon();

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
#define MOCGPU_THROW(code, msg) throw ::mocgpu::Error((code), (msg))

// ---- fuzzy floating point comparisons -------------------------------------
// ULP distance with MOCC's sign folding (it folds negatives with a 2^31
// offset on a 64-bit integer; kept as is so tie-breaks match).
inline bool fp_equiv_ulp(double a, double b)
{
    int64_t ia, ib;
    static_assert(sizeof(double) == sizeof(int64_t), "double size");
    __builtin_memcpy(&ia, &a, 8);
    __builtin_memcpy(&ib, &b, 8);
    if (ia < 0) ia = (int64_t)0x80000000 - ia;
    if (ib < 0) ib = (int64_t)0x80000000 - ib;
    int64_t d = ia - ib;
    if (d < 0) d = -d;
    return d < 200;
}
inline bool fp_equiv_abs(double a, double b) { return std::fabs(a - b) < kFuzz; }
inline bool fp_equiv_rel(double a, double b) { return std::fabs(a - b) / std::fabs(a) < kFuzz; }
inline bool fp_equiv(double a, double b)
{
    if (fp_equiv_abs(a, b)) return true;
    if ((a < 0.0) != (b < 0.0)) return false;
    return fp_equiv_ulp(a, b);
}
// "l is sufficiently less than r", for lower_bound over sorted boundaries.
inline bool fuzzy_lt(double l, double r) { return (l - r) / std::fabs(r) < -kFuzz; }

// ---- points ----------------------------------------------------------------
struct Point2 {
    double x = 0.0, y = 0.0;
    bool ok = false;
    Point2() = default;
    Point2(double x_, double y_) : x(x_), y(y_), ok(true) {}
    double distance(const Point2 &p) const
    {
        return std::sqrt((x - p.x) * (x - p.x) + (y - p.y) * (y - p.y));
    }
    // Ordering is by y only: every traced ray runs upward (octants 1-2).
    bool operator<(const Point2 &o) const { return y < o.y; }
    bool operator==(const Point2 &o) const { return fp_equiv(x, o.x) && fp_equiv(y, o.y); }
    Point2 operator-(const Point2 &o) const { return Point2(x - o.x, y - o.y); }
    // Angle from +x axis folded into [0, 2pi].
    double alpha() const { return (y > 0.0) ? std::atan2(y, x) : std::atan2(y, x) + kTwoPi; }
};
inline Point2 midpoint(const Point2 &a, const Point2 &b)
{
    return Point2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
}

struct Line {
    Point2 p1, p2;
    Line() = default;
    Line(Point2 a, Point2 b) : p1(a), p2(b) {}
};
struct Circle {
    Point2 c;
    double r = 0.0;
    Circle(Point2 c_, double r_) : c(c_), r(r_) {}
};

// Segment/circle crossing; returns the number of crossings strictly inside
// the segment (0 for a miss or an exact tangent).
inline int intersect(const Line &l, const Circle &circ, Point2 &p1, Point2 &p2)
{
    double u1 = l.p2.x - l.p1.x, u2 = l.p2.y - l.p1.y;
    double w1 = l.p1.x - circ.c.x, w2 = l.p1.y - circ.c.y;
    double b = w1 * u1 + w2 * u2;
    double c = w1 * w1 + w2 * w2 - circ.r * circ.r;
    if ((c > 0.0) & (b > 0.0)) return 0;
    double a = u1 * u1 + u2 * u2;
    double disc = b * b - a * c;
    if (disc < 0.0) return 0;
    if (fp_equiv_rel(disc, 0.0)) return 0;
    int ret = 0;
    double ra = 1.0 / a;
    disc = std::sqrt(disc);
    double t1 = (-b - disc) * ra;
    double t2 = (-b + disc) * ra;
    if ((0.0 < t1) & (t1 < 1.0)) {
        p1 = l.p1;
        p1.x += u1 * t1;
        p1.y += u2 * t1;
        p1.ok = true;
        ret++;
    }
    if ((0.0 < t2) & (t2 < 1.0)) {
        Point2 &dst = (ret == 0) ? p1 : p2;
        dst = l.p1;
        dst.x += u1 * t2;
        dst.y += u2 * t2;
        dst.ok = true;
        ret++;
    }
    return ret;
}

// Segment/segment crossing; the point is computed on l1 (the mesh line), so a
// crossing of an axis-aligned mesh line keeps that line's exact coordinate.
inline int intersect(const Line &l1, const Line &l2, Point2 &p)
{
    double u1 = l1.p2.x - l1.p1.x, u2 = l1.p2.y - l1.p1.y;
    double v1 = l2.p2.x - l2.p1.x, v2 = l2.p2.y - l2.p1.y;
    double w1 = l1.p1.x - l2.p1.x, w2 = l1.p1.y - l2.p1.y;
    double d = u1 * v2 - u2 * v1;
    double s = v1 * w2 - v2 * w1;
    double t = u1 * w2 - u2 * w1;
    s = s / d;
    t = t / d;
    if ((0.0 <= s) & (s <= 1.0) & (0.0 <= t) & (t <= 1.0)) {
        p = l1.p1;
        p.x += s * u1;
        p.y += s * u2;
        p.ok = true;
        return 1;
    }
    return 0;
}

// ---- directions -------------------------------------------------------------
struct Direction {
    double ox = 0, oy = 0, oz = 0, alpha = 0, theta = 0, rsintheta = 0;
    Direction() = default;
    // From azimuthal/polar angles (extended precision like the reference).
    static Direction from_angles(double alpha, double theta)
    {
        Direction d;
        d.alpha = alpha;
        d.theta = theta;
        long double st = std::sin((long double)theta);
        d.ox = (double)(st * std::cos((long double)alpha));
        d.oy = (double)(st * std::sin((long double)alpha));
        d.oz = (double)std::cos((long double)theta);
        d.rsintheta = (double)(1.0L / st);
        return d;
    }
    // From direction cosines.
    static Direction from_cosines(double ox, double oy, double oz)
    {
        Direction d;
        d.ox = ox;
        d.oy = oy;
        d.oz = oz;
        long double th = std::acos((long double)oz);
        d.theta = (double)th;
        d.alpha = (double)std::acos((long double)ox / std::sin(th));
        if (oy < 0.0) d.alpha = kTwoPi - d.alpha;
        d.rsintheta = (double)(1.0L / std::sin(th));
        return d;
    }
    Direction to_octant(int oct) const
    {
        double ax = std::fabs(ox), ay = std::fabs(oy), az = std::fabs(oz);
        switch (oct) {
        case 1: return from_cosines(ax, ay, az);
        case 2: return from_cosines(-ax, ay, az);
        case 3: return from_cosines(-ax, -ay, az);
        case 4: return from_cosines(ax, -ay, az);
        case 5: return from_cosines(ax, ay, -az);
        case 6: return from_cosines(-ax, ay, -az);
        case 7: return from_cosines(-ax, -ay, -az);
        case 8: return from_cosines(ax, -ay, -az);
        }
        MOCGPU_THROW(1, "invalid octant");
    }
};

struct Angle : Direction {
    double weight = 0.0;
    Angle() = default;
    Angle(const Direction &d, double w) : Direction(d), weight(w) {}
    Angle to_octant(int oct) const { return Angle(Direction::to_octant(oct), weight); }
    void modify_alpha(double a)
    {
        Direction d = Direction::from_angles(a, theta);
        static_cast<Direction &>(*this) = d;
    }
};

// Axis-aligned box; intersect() returns the exit point of a ray from p.
// The candidate test keeps MOCC's form (signed distance compared against the
// running |d| minimum; strict interior tests on the other coordinate).
struct Box {
    Point2 lo, hi;
    Box() = default;
    Box(Point2 a, Point2 b) : lo(a), hi(b) {}
    Point2 intersect(Point2 p, double alpha) const
    {
        double ox = std::cos(alpha), oy = std::sin(alpha);
        double dmin = 1.0e12, d, x, y;
        Point2 out;
        x = lo.x;
        d = (lo.x - p.x) / ox;
        y = p.y + oy * d;
        if ((std::fabs(d) > kFuzz) && (d < dmin) && (y > lo.y) && (y < hi.y)) {
            dmin = std::fabs(d);
            out = Point2(x, y);
        }
        x = hi.x;
        d = (hi.x - p.x) / ox;
        y = p.y + oy * d;
        if ((std::fabs(d) > kFuzz) && (d < dmin) && (y > lo.y) && (y < hi.y)) {
            dmin = std::fabs(d);
            out = Point2(x, y);
        }
        y = lo.y;
        d = (lo.y - p.y) / oy;
        x = p.x + ox * d;
        if ((std::fabs(d) > kFuzz) && (d < dmin) && (x > lo.x) && (x < hi.x)) {
            dmin = std::fabs(d);
            out = Point2(x, y);
        }
        y = hi.y;
        d = (hi.y - p.y) / oy;
        x = p.x + ox * d;
        if ((std::fabs(d) > kFuzz) && (d < dmin) && (x > lo.x) && (x < hi.x)) {
            dmin = std::fabs(d);
            out = Point2(x, y);
        }
        return out;
    }
};

// Surfaces and normals, numbered as in MOCC (src/core/constants.hpp:34-64).
enum Surface : int { EAST = 0, NORTH = 1, WEST = 2, SOUTH = 3, TOP = 4, BOTTOM = 5, INTERNAL = 6, INVALID = 7 };
enum Normal : int { X_NORM = 0, Y_NORM = 1, Z_NORM = 2 };
enum class BoundaryType : int { VACUUM = 0, REFLECT = 1, PARALLEL = 2, PERIODIC = 3, PRESCRIBED = 4, INVALID = 5 };

inline Normal surface_normal_of(Surface s)
{
    switch (s) {
    case EAST:
    case WEST: return X_NORM;
    case NORTH:
    case SOUTH: return Y_NORM;
    case TOP:
    case BOTTOM: return Z_NORM;
    default: MOCGPU_THROW(1, "unsupported surface");
    }
}

} // namespace mocgpu
