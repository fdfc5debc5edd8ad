// motion.h -- pose of a body in prescribed rigid motion (no reference
// counterpart: the reference claims moving boundaries, README.md:7,11, but
// has no code for them).
//
// Angles are carried in turns (1 turn = 2 pi).  Sine and cosine of 2 pi x are
// formed by reduction of x to [0, 1/8] turn (exact: x - floor(x), the
// quadrant and the octant mirror are exact operations) and the Taylor series
// of sin and cos on [0, pi/4] up to degree 19 (truncation below 1e-19).
// Every operation is rounded on its own (host code is compiled with
// -ffp-contract=off, device code that uses this header with -fmad=false), so
// the host, the device and a CPU restatement that performs the same operations
// produce the same bits.
#pragma once
#include <cmath>

#include "../../include/immerseflow_gb300.h"
#include "ifx_dev.h"

namespace ifx {

IFX_HD inline void sincos_turns(double x, double* s, double* c) {
    const double r = x - floor(x);           // [0, 1)
    const double r4 = r * 4.0;               // exact
    const int q = (int)r4;                   // quadrant 0..3
    double f = r4 - (double)q;               // [0, 1) of the quadrant, exact
    const bool mirror = f > 0.5;
    if (mirror) f = 1.0 - f;                 // exact
    const double a = f * (3.14159265358979323846 / 2.0);  // [0, pi/4]
    const double a2 = a * a;
    double ps = 1.0 / 121645100408832000.0;  // 1/19!
    ps = 1.0 / 355687428096000.0 - a2 * ps;  // 1/17!
    ps = 1.0 / 1307674368000.0 - a2 * ps;    // 1/15!
    ps = 1.0 / 6227020800.0 - a2 * ps;       // 1/13!
    ps = 1.0 / 39916800.0 - a2 * ps;         // 1/11!
    ps = 1.0 / 362880.0 - a2 * ps;           // 1/9!
    ps = 1.0 / 5040.0 - a2 * ps;             // 1/7!
    ps = 1.0 / 120.0 - a2 * ps;              // 1/5!
    ps = 1.0 / 6.0 - a2 * ps;                // 1/3!
    ps = 1.0 - a2 * ps;
    double pc = 1.0 / 20922789888000.0;      // 1/16!
    pc = 1.0 / 87178291200.0 - a2 * pc;      // 1/14!
    pc = 1.0 / 479001600.0 - a2 * pc;        // 1/12!
    pc = 1.0 / 3628800.0 - a2 * pc;          // 1/10!
    pc = 1.0 / 40320.0 - a2 * pc;            // 1/8!
    pc = 1.0 / 720.0 - a2 * pc;              // 1/6!
    pc = 1.0 / 24.0 - a2 * pc;               // 1/4!
    pc = 1.0 / 2.0 - a2 * pc;                // 1/2!
    pc = 1.0 - a2 * pc;
    double sa = a * ps, ca = pc;             // sin, cos of the reduced angle
    if (mirror) {                            // angle = pi/2 - a within the quadrant
        const double t = sa;
        sa = ca;
        ca = t;
    }
    switch (q) {                             // rotate by q quarter turns
        case 0: *s = sa; *c = ca; break;
        case 1: *s = ca; *c = -sa; break;
        case 2: *s = -sa; *c = -ca; break;
        default: *s = -ca; *c = sa; break;
    }
}

// Motion constants of an instance (angles in turns, w = 2 pi f) from its
// configuration; the initial pose is the configured one.
struct MotionDef {
    double x0, y0, th0, u, v, ax, ay, ath, f, w, phx, phy, pha;
};

inline MotionDef motion_def(const ifx_config& c) {
    MotionDef m;
    m.x0 = c.body_cx;
    m.y0 = c.body_cy;
    m.th0 = c.body_angle_deg / 360.0;
    m.u = c.motion_u;
    m.v = c.motion_v;
    m.ax = c.motion_amp_x;
    m.ay = c.motion_amp_y;
    m.ath = c.motion_amp_deg / 360.0;
    m.f = c.motion_freq;
    m.w = (2.0 * 3.14159265358979323846) * c.motion_freq;
    m.phx = c.motion_phase_x / 360.0;
    m.phy = c.motion_phase_y / 360.0;
    m.pha = c.motion_phase_deg / 360.0;
    return m;
}

struct Pose {
    double x, y, c, s;  // centre, cos and sin of the angle
    double u, v, w;     // velocity of the centre, rotation rate (rad/time)
};

// Pose at time t: see IFX_MOTION_PRESCRIBED.
IFX_HD inline Pose pose_at(double x0, double y0, double th0, double u, double v, double ax, double ay, double ath,
                           double f, double w, double phx, double phy, double pha, double t) {
    const double ft = f * t;
    double s0, c0, s1, c1;
    Pose p;
    sincos_turns(phx, &s0, &c0);
    sincos_turns(ft + phx, &s1, &c1);
    p.x = (x0 + u * t) + ax * (s1 - s0);
    p.u = u + (ax * w) * c1;
    sincos_turns(phy, &s0, &c0);
    sincos_turns(ft + phy, &s1, &c1);
    p.y = (y0 + v * t) + ay * (s1 - s0);
    p.v = v + (ay * w) * c1;
    sincos_turns(pha, &s0, &c0);
    sincos_turns(ft + pha, &s1, &c1);
    const double th = th0 + ath * (s1 - s0);
    p.w = ((ath * (2.0 * 3.14159265358979323846)) * w) * c1;
    sincos_turns(th, &p.s, &p.c);
    return p;
}

}  // namespace ifx
