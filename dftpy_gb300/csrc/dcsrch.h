// More-Thuente line search (MINPACK-2 dcsrch / dcstep algorithm, Moré &
// Thuente, ACM TOMS 20 (1994) 286-307) as a reverse-communication state
// machine.  Drives the rotation-angle search of the density optimiser the
// same way dftpy's LineSearchDcsrch2 drives minpack2.dcsrch
// (src/dftpy/math_utils.py:76-106).
#pragma once
#include <math.h>

enum DcsTask { DCS_START = 0, DCS_FG = 1, DCS_CONV = 2, DCS_WARN = 3, DCS_ERROR = 4 };

struct Dcsrch {
  double ftol, gtol, xtol, stpmin, stpmax;
  int brackt, stage;
  double finit, ginit, gtest, width, width1;
  double stx, fx, gx, sty, fy, gy, stmin, stmax;
};

static inline void dcs_init(Dcsrch& s, double ftol, double gtol, double xtol, double stpmin, double stpmax) {
  s.ftol = ftol; s.gtol = gtol; s.xtol = xtol; s.stpmin = stpmin; s.stpmax = stpmax;
}

static inline void dcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
                          double fp, double dp, int& brackt, double stpmin, double stpmax) {
  const double sgnd = dp * (dx / fabs(dx));
  double stpf;
  if (fp > fx) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp, r = p / q;
    const double stpc = stx + r * (stp - stx);
    const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
    stpf = (fabs(stpc - stx) <= fabs(stpq - stx)) ? stpc : stpc + (stpq - stpc) / 2.0;
    brackt = 1;
  } else if (sgnd < 0.0) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx, r = p / q;
    const double stpc = stp + r * (stx - stp);
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    stpf = (fabs(stpc - stp) > fabs(stpq - stp)) ? stpc : stpq;
    brackt = 1;
  } else if (fabs(dp) < fabs(dx)) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
    double gamma = s * sqrt(fmax(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma, r = p / q;
    double stpc;
    if (r < 0.0 && gamma != 0.0) stpc = stp + r * (stx - stp);
    else if (stp > stx) stpc = stpmax;
    else stpc = stpmin;
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) {
      stpf = (fabs(stpc - stp) < fabs(stpq - stp)) ? stpc : stpq;
      if (stp > stx) stpf = fmin(stp + 0.66 * (sty - stp), stpf);
      else stpf = fmax(stp + 0.66 * (sty - stp), stpf);
    } else {
      stpf = (fabs(stpc - stp) > fabs(stpq - stp)) ? stpc : stpq;
      stpf = fmin(stpmax, stpf);
      stpf = fmax(stpmin, stpf);
    }
  } else {
    if (brackt) {
      const double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
      const double s = fmax(fabs(theta), fmax(fabs(dy), fabs(dp)));
      double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dy, r = p / q;
      stpf = stp + r * (sty - stp);
    } else if (stp > stx) {
      stpf = stpmax;
    } else {
      stpf = stpmin;
    }
  }
  if (fp > fx) {
    sty = stp; fy = fp; dy = dp;
  } else {
    if (sgnd < 0.0) { sty = stx; fy = fx; dy = dx; }
    stx = stp; fx = fp; dx = dp;
  }
  stp = stpf;
}

// One call of the state machine; returns the new task (stp updated in place).
static inline int dcs_step(Dcsrch& s, double& stp, double f, double g, int task) {
  const double xtrapl = 1.1, xtrapu = 4.0, p5 = 0.5, p66 = 0.66;
  if (task == DCS_START) {
    if (stp < s.stpmin || stp > s.stpmax || g >= 0.0 || s.ftol < 0.0 || s.gtol < 0.0 || s.xtol < 0.0 ||
        s.stpmin < 0.0 || s.stpmax < s.stpmin)
      return DCS_ERROR;
    s.brackt = 0; s.stage = 1; s.finit = f; s.ginit = g; s.gtest = s.ftol * g;
    s.width = s.stpmax - s.stpmin; s.width1 = s.width / p5;
    s.stx = 0.0; s.fx = f; s.gx = g; s.sty = 0.0; s.fy = f; s.gy = g;
    s.stmin = 0.0; s.stmax = stp + xtrapu * stp;
    return DCS_FG;
  }
  const double ftest = s.finit + stp * s.gtest;
  if (s.stage == 1 && f <= ftest && g >= 0.0) s.stage = 2;
  int t = -1;
  if (s.brackt && (stp <= s.stmin || stp >= s.stmax)) t = DCS_WARN;
  if (s.brackt && s.stmax - s.stmin <= s.xtol * s.stmax) t = DCS_WARN;
  if (stp == s.stpmax && f <= ftest && g <= s.gtest) t = DCS_WARN;
  if (stp == s.stpmin && (f > ftest || g >= s.gtest)) t = DCS_WARN;
  if (f <= ftest && fabs(g) <= s.gtol * (-s.ginit)) t = DCS_CONV;
  if (t >= 0) return t;
  if (s.stage == 1 && f <= s.fx && f > ftest) {
    const double gt = s.gtest;
    double fm = f - stp * gt, fxm = s.fx - s.stx * gt, fym = s.fy - s.sty * gt;
    double gm = g - gt, gxm = s.gx - gt, gym = s.gy - gt;
    dcstep(s.stx, fxm, gxm, s.sty, fym, gym, stp, fm, gm, s.brackt, s.stmin, s.stmax);
    s.fx = fxm + s.stx * gt; s.fy = fym + s.sty * gt;
    s.gx = gxm + gt; s.gy = gym + gt;
  } else {
    dcstep(s.stx, s.fx, s.gx, s.sty, s.fy, s.gy, stp, f, g, s.brackt, s.stmin, s.stmax);
  }
  if (s.brackt) {
    if (fabs(s.sty - s.stx) >= p66 * s.width1) stp = s.stx + p5 * (s.sty - s.stx);
    s.width1 = s.width;
    s.width = fabs(s.sty - s.stx);
    s.stmin = fmin(s.stx, s.sty);
    s.stmax = fmax(s.stx, s.sty);
  } else {
    s.stmin = stp + xtrapl * (stp - s.stx);
    s.stmax = stp + xtrapu * (stp - s.stx);
  }
  stp = fmax(stp, s.stpmin);
  stp = fmin(stp, s.stpmax);
  if ((s.brackt && (stp <= s.stmin || stp >= s.stmax)) || (s.brackt && s.stmax - s.stmin <= s.xtol * s.stmax))
    stp = s.stx;
  return DCS_FG;
}
