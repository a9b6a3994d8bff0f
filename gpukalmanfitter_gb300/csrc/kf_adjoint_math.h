// kf_adjoint_math.h — vector-Jacobian products (reverse-mode derivatives) of
// the FP64 fit primitives, for the chi2 adjoint.
//
// Every primitive comes as a pair: xxxFwd evaluates the forward formula (the
// same mathematics as the fit kernel's FP64 form, restated as a pure
// function), xxxVjp takes the adjoints of the outputs and ADDS the adjoints
// of the inputs into the caller's accumulators.  Uniform field only: the
// field B = scale * B0 does not depend on position, so the RK stages depend
// on the direction, q/p, the step and B.
//
// Host and device: the CPU tests check each product against central finite
// differences of the forward formula.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define KF_HD __host__ __device__ __forceinline__
#else
#define KF_HD inline
#endif

namespace kfa {

// 1 / sqrt(a): the device's reciprocal square root (one MUFU seed and Newton
// steps instead of a square root and a division)
KF_HD double rsqrtD(double a) {
#ifdef __CUDA_ARCH__
  return rsqrt(a);
#else
  return 1. / std::sqrt(a);
#endif
}

// sine and cosine of one angle (one argument reduction on the device)
KF_HD void sinCos(double x, double &sn, double &cs) {
#ifdef __CUDA_ARCH__
  sincos(x, &sn, &cs);
#else
  sn = std::sin(x);
  cs = std::cos(x);
#endif
}

KF_HD void cross(const double a[3], const double b[3], double r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
KF_HD double dot(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
// adjoint of r = a x b: abar += b x rbar, bbar += rbar x a
KF_HD void crossVjp(const double a[3], const double b[3], const double rb[3], double ab[3],
                    double bb[3]) {
  double t[3];
  cross(b, rb, t);
  for (int i = 0; i < 3; ++i) ab[i] += t[i];
  cross(rb, a, t);
  for (int i = 0; i < 3; ++i) bb[i] += t[i];
}

// ---------------------------------------------------------------------------
// RK4 stages and error estimate (EigenStepper.ipp:243-269, uniform field)
//   k1 = q (d x B), k2 = q ((d + h/2 k1) x B), k3 = q ((d + h/2 k2) x B),
//   k4 = q ((d + h k3) x B),  err = max(h^2 |k1 - k2 - k3 + k4|_1, 1e-20)
// ---------------------------------------------------------------------------
struct Stages {
  double k1[3], k2[3], k3[3], k4[3];
  double u2[3], u3[3], u4[3]; // stage arguments d + a k
  double c1[3], c2[3], c3[3], c4[3];
  double dl[3]; // k1 - k2 - k3 + k4
  double err;
};

KF_HD void stagesFwd(const double d[3], double q, double h, const double B[3], Stages &s) {
  const double a = h * 0.5;
  cross(d, B, s.c1);
  for (int i = 0; i < 3; ++i) s.k1[i] = q * s.c1[i];
  for (int i = 0; i < 3; ++i) s.u2[i] = d[i] + a * s.k1[i];
  cross(s.u2, B, s.c2);
  for (int i = 0; i < 3; ++i) s.k2[i] = q * s.c2[i];
  for (int i = 0; i < 3; ++i) s.u3[i] = d[i] + a * s.k2[i];
  cross(s.u3, B, s.c3);
  for (int i = 0; i < 3; ++i) s.k3[i] = q * s.c3[i];
  for (int i = 0; i < 3; ++i) s.u4[i] = d[i] + h * s.k3[i];
  cross(s.u4, B, s.c4);
  for (int i = 0; i < 3; ++i) s.k4[i] = q * s.c4[i];
  double e = 0.;
  for (int i = 0; i < 3; ++i) {
    s.dl[i] = s.k1[i] - s.k2[i] - s.k3[i] + s.k4[i];
    e += fabs(s.dl[i]);
  }
  e *= h * h;
  s.err = e < 1e-20 ? 1e-20 : e;
}

// kb1..kb4 are consumed (modified); errb is the adjoint of err
KF_HD void stagesVjp(const double d[3], double q, double h, const double B[3], const Stages &s,
                     double kb1[3], double kb2[3], double kb3[3], double kb4[3], double errb,
                     double db[3], double &qb, double &hb, double Bb[3]) {
  const double a = h * 0.5;
  double ab = 0.;
  if (errb != 0. && s.err > 1e-20) {
    double l1 = 0.;
    for (int i = 0; i < 3; ++i) l1 += fabs(s.dl[i]);
    hb += errb * 2. * h * l1;
    for (int i = 0; i < 3; ++i) {
      const double g = errb * h * h * (s.dl[i] > 0. ? 1. : (s.dl[i] < 0. ? -1. : 0.));
      kb1[i] += g;
      kb2[i] -= g;
      kb3[i] -= g;
      kb4[i] += g;
    }
  }
  double cb[3], ub[3];
  // k4 = q c4, c4 = u4 x B, u4 = d + h k3
  for (int i = 0; i < 3; ++i) {
    qb += kb4[i] * s.c4[i];
    cb[i] = q * kb4[i];
    ub[i] = 0.;
  }
  crossVjp(s.u4, B, cb, ub, Bb);
  for (int i = 0; i < 3; ++i) {
    db[i] += ub[i];
    hb += ub[i] * s.k3[i];
    kb3[i] += h * ub[i];
  }
  // k3 = q c3, c3 = u3 x B, u3 = d + a k2
  for (int i = 0; i < 3; ++i) {
    qb += kb3[i] * s.c3[i];
    cb[i] = q * kb3[i];
    ub[i] = 0.;
  }
  crossVjp(s.u3, B, cb, ub, Bb);
  for (int i = 0; i < 3; ++i) {
    db[i] += ub[i];
    ab += ub[i] * s.k2[i];
    kb2[i] += a * ub[i];
  }
  // k2 = q c2, c2 = u2 x B, u2 = d + a k1
  for (int i = 0; i < 3; ++i) {
    qb += kb2[i] * s.c2[i];
    cb[i] = q * kb2[i];
    ub[i] = 0.;
  }
  crossVjp(s.u2, B, cb, ub, Bb);
  for (int i = 0; i < 3; ++i) {
    db[i] += ub[i];
    ab += ub[i] * s.k1[i];
    kb1[i] += a * ub[i];
  }
  // k1 = q c1, c1 = d x B
  for (int i = 0; i < 3; ++i) {
    qb += kb1[i] * s.c1[i];
    cb[i] = q * kb1[i];
  }
  crossVjp(d, B, cb, db, Bb);
  hb += 0.5 * ab;
}

// ---------------------------------------------------------------------------
// Accepted step: state update (EigenStepper.ipp:300-330)
//   pos' = pos + h d + h^2/6 (k1 + k2 + k3)
//   w = d + h/6 (k1 + 2 k2 + 2 k3 + k4),  d' = w / |w|,  t' = t + h dtds
// ---------------------------------------------------------------------------
struct Moved {
  double pos[3], dir[3], t;
  double w[3], n;
};

KF_HD void acceptFwd(const double pos[3], const double d[3], double t, double h, double dtds,
                     const Stages &s, Moved &m) {
  const double hh6 = h * h / 6., h6 = h / 6.;
  for (int i = 0; i < 3; ++i) {
    m.pos[i] = pos[i] + (h * d[i] + hh6 * (s.k1[i] + s.k2[i] + s.k3[i]));
    m.w[i] = d[i] + h6 * (s.k1[i] + 2. * (s.k2[i] + s.k3[i]) + s.k4[i]);
  }
  m.n = sqrt(dot(m.w, m.w));
  for (int i = 0; i < 3; ++i) m.dir[i] = m.w[i] / m.n;
  m.t = t + h * dtds;
}

KF_HD void acceptVjp(const double d[3], double h, double dtds, const Stages &s, const Moved &m,
                     const double posb_[3], const double dirb_[3], double tb_, double posb[3],
                     double db[3], double &tb, double &hb, double &dtdsb, double kb1[3],
                     double kb2[3], double kb3[3], double kb4[3]) {
  const double hh6 = h * h / 6., h6 = h / 6.;
  tb += tb_;
  hb += tb_ * dtds;
  dtdsb += tb_ * h;
  // d' = w / n
  const double pr = dot(m.dir, dirb_);
  double wb[3];
  for (int i = 0; i < 3; ++i) wb[i] = (dirb_[i] - m.dir[i] * pr) / m.n;
  for (int i = 0; i < 3; ++i) {
    db[i] += wb[i];
    const double ksum = s.k1[i] + 2. * (s.k2[i] + s.k3[i]) + s.k4[i];
    hb += wb[i] * ksum / 6.;
    kb1[i] += h6 * wb[i];
    kb2[i] += 2. * h6 * wb[i];
    kb3[i] += 2. * h6 * wb[i];
    kb4[i] += h6 * wb[i];
  }
  for (int i = 0; i < 3; ++i) {
    posb[i] += posb_[i];
    db[i] += h * posb_[i];
    const double k3s = s.k1[i] + s.k2[i] + s.k3[i];
    hb += posb_[i] * (d[i] + h / 3. * k3s);
    kb1[i] += hh6 * posb_[i];
    kb2[i] += hh6 * posb_[i];
    kb3[i] += hh6 * posb_[i];
  }
}

// ---------------------------------------------------------------------------
// Step transport matrix (EigenStepper.ipp:50-124) on its non-zero blocks and
// the Jacobian accumulation J <- D J (EigenStepper.ipp:312-318).
//   T1 = q [.,B],  T(n+1)[:,j] = q (e_j + hh Tn[:,j]) x B  (hh = h/2, h/2, h)
//   L1 = d x B,  L(n+1) = u(n+1) x B + q hh (Ln x B)
//   DA = h (I + h/6 (T1 + T2 + T3)),  DB = I + h/6 (T1 + 2 T2 + 2 T3 + T4)
//   Da = h^2/6 (L1 + L2 + L3),  Dc = h/6 (L1 + 2 L2 + 2 L3 + L4),  D37 = h d37
// ---------------------------------------------------------------------------
struct DMat {
  double DA[3][3], DB[3][3], Da[3], Dc[3], D37;
};
struct TransportTmp {
  double T[4][3][3]; // T1..T4
  double L[4][3];    // dk1dL..dk4dL
};
// transport Jacobian blocks: [[I, 0, A, a], [0, 1, 0, b], [0, 0, B, c], [0, 0, 0, 1]]
struct JT {
  double A[3][3], a[3], b, B[3][3], c[3];
};

KF_HD void jtIdentity(JT &J) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      J.A[i][j] = 0.;
      J.B[i][j] = (i == j) ? 1. : 0.;
    }
    J.a[i] = 0.;
    J.c[i] = 0.;
  }
  J.b = 0.;
}
KF_HD void jtZero(JT &J) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) J.A[i][j] = J.B[i][j] = 0.;
    J.a[i] = J.c[i] = 0.;
  }
  J.b = 0.;
}
KF_HD void dmZero(DMat &D) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) D.DA[i][j] = D.DB[i][j] = 0.;
    D.Da[i] = D.Dc[i] = 0.;
  }
  D.D37 = 0.;
}

KF_HD void tNext(const double Tp[3][3], double hh, double q, const double B[3], double To[3][3]) {
  for (int j = 0; j < 3; ++j) {
    double col[3], r[3];
    for (int i = 0; i < 3; ++i) col[i] = ((i == j) ? 1. : 0.) + hh * Tp[i][j];
    cross(col, B, r);
    for (int i = 0; i < 3; ++i) To[i][j] = q * r[i];
  }
}
KF_HD void tNextVjp(const double Tp[3][3], double hh, double q, const double B[3],
                    const double Tob[3][3], double Tpb[3][3], double &hhb, double &qb,
                    double Bb[3]) {
  for (int j = 0; j < 3; ++j) {
    double col[3], r[3], rb[3], colb[3] = {0., 0., 0.};
    for (int i = 0; i < 3; ++i) col[i] = ((i == j) ? 1. : 0.) + hh * Tp[i][j];
    cross(col, B, r);
    for (int i = 0; i < 3; ++i) {
      qb += Tob[i][j] * r[i];
      rb[i] = q * Tob[i][j];
    }
    crossVjp(col, B, rb, colb, Bb);
    for (int i = 0; i < 3; ++i) {
      Tpb[i][j] += hh * colb[i];
      hhb += colb[i] * Tp[i][j];
    }
  }
}

KF_HD void transportFwd(const double d[3], double q, double h, double d37, const double B[3],
                        const Stages &s, DMat &D, TransportTmp &X) {
  double(&T1)[3][3] = X.T[0];
  T1[0][0] = 0.;
  T1[0][1] = q * B[2];
  T1[0][2] = q * -B[1];
  T1[1][0] = q * -B[2];
  T1[1][1] = 0.;
  T1[1][2] = q * B[0];
  T1[2][0] = q * B[1];
  T1[2][1] = q * -B[0];
  T1[2][2] = 0.;
  const double a = h * 0.5;
  tNext(X.T[0], a, q, B, X.T[1]);
  tNext(X.T[1], a, q, B, X.T[2]);
  tNext(X.T[2], h, q, B, X.T[3]);
  double cc[3];
  cross(d, B, X.L[0]);
  cross(X.L[0], B, cc);
  for (int i = 0; i < 3; ++i) X.L[1][i] = s.c2[i] + (q * a) * cc[i];
  cross(X.L[1], B, cc);
  for (int i = 0; i < 3; ++i) X.L[2][i] = s.c3[i] + (q * a) * cc[i];
  cross(X.L[2], B, cc);
  for (int i = 0; i < 3; ++i) X.L[3][i] = s.c4[i] + (q * h) * cc[i];
  const double h6 = h / 6.;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      const double v = ((i == j) ? 1. : 0.) + h6 * (X.T[0][i][j] + X.T[1][i][j] + X.T[2][i][j]);
      D.DA[i][j] = v * h;
      D.DB[i][j] = ((i == j) ? 1. : 0.) +
                   h6 * (X.T[0][i][j] + 2. * (X.T[1][i][j] + X.T[2][i][j]) + X.T[3][i][j]);
    }
    D.Da[i] = (h * h) / 6. * (X.L[0][i] + X.L[1][i] + X.L[2][i]);
    D.Dc[i] = h6 * (X.L[0][i] + 2. * (X.L[1][i] + X.L[2][i]) + X.L[3][i]);
  }
  D.D37 = h * d37;
}

// adjoint of D -> d, q, h, d37, B and the stage values k1, k2, k3 (through
// the stage arguments u2 = d + h/2 k1, u3 = d + h/2 k2, u4 = d + h k3)
KF_HD void transportVjp(const double d[3], double q, double h, double d37, const double B[3],
                        const Stages &s, const TransportTmp &X, const DMat &Db, double db[3],
                        double &qb, double &hb, double &d37b, double Bb[3], double kb1[3],
                        double kb2[3], double kb3[3]) {
  const double a = h * 0.5, h6 = h / 6.;
  double h6b = 0., ab = 0.;
  double Tb[4][3][3], Lb[4][3];
  for (int n = 0; n < 4; ++n)
    for (int i = 0; i < 3; ++i) {
      Lb[n][i] = 0.;
      for (int j = 0; j < 3; ++j) Tb[n][i][j] = 0.;
    }
  hb += Db.D37 * d37;
  d37b += Db.D37 * h;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      const double S = X.T[0][i][j] + X.T[1][i][j] + X.T[2][i][j];
      const double v = ((i == j) ? 1. : 0.) + h6 * S;
      hb += Db.DA[i][j] * v;
      const double vb = Db.DA[i][j] * h;
      h6b += vb * S;
      Tb[0][i][j] += h6 * vb;
      Tb[1][i][j] += h6 * vb;
      Tb[2][i][j] += h6 * vb;
      const double S2 = X.T[0][i][j] + 2. * (X.T[1][i][j] + X.T[2][i][j]) + X.T[3][i][j];
      h6b += Db.DB[i][j] * S2;
      Tb[0][i][j] += h6 * Db.DB[i][j];
      Tb[1][i][j] += 2. * h6 * Db.DB[i][j];
      Tb[2][i][j] += 2. * h6 * Db.DB[i][j];
      Tb[3][i][j] += h6 * Db.DB[i][j];
    }
    const double Ls = X.L[0][i] + X.L[1][i] + X.L[2][i];
    hb += Db.Da[i] * (h / 3.) * Ls;
    const double c6 = (h * h) / 6.;
    Lb[0][i] += c6 * Db.Da[i];
    Lb[1][i] += c6 * Db.Da[i];
    Lb[2][i] += c6 * Db.Da[i];
    const double Lc = X.L[0][i] + 2. * (X.L[1][i] + X.L[2][i]) + X.L[3][i];
    h6b += Db.Dc[i] * Lc;
    Lb[0][i] += h6 * Db.Dc[i];
    Lb[1][i] += 2. * h6 * Db.Dc[i];
    Lb[2][i] += 2. * h6 * Db.Dc[i];
    Lb[3][i] += h6 * Db.Dc[i];
  }
  hb += h6b / 6.;
  // L4 = u4 x B + (q h) (L3 x B)
  {
    double ub[3] = {0., 0., 0.}, r[3], rb[3];
    crossVjp(s.u4, B, Lb[3], ub, Bb);
    for (int i = 0; i < 3; ++i) {
      db[i] += ub[i];
      hb += ub[i] * s.k3[i];
      kb3[i] += h * ub[i];
    }
    cross(X.L[2], B, r);
    const double sc = q * h;
    const double scb = dot(Lb[3], r);
    qb += scb * h;
    hb += scb * q;
    for (int i = 0; i < 3; ++i) rb[i] = sc * Lb[3][i];
    crossVjp(X.L[2], B, rb, Lb[2], Bb);
  }
  // L3 = u3 x B + (q a) (L2 x B)
  {
    double ub[3] = {0., 0., 0.}, r[3], rb[3];
    crossVjp(s.u3, B, Lb[2], ub, Bb);
    for (int i = 0; i < 3; ++i) {
      db[i] += ub[i];
      ab += ub[i] * s.k2[i];
      kb2[i] += a * ub[i];
    }
    cross(X.L[1], B, r);
    const double sc = q * a;
    const double scb = dot(Lb[2], r);
    qb += scb * a;
    ab += scb * q;
    for (int i = 0; i < 3; ++i) rb[i] = sc * Lb[2][i];
    crossVjp(X.L[1], B, rb, Lb[1], Bb);
  }
  // L2 = u2 x B + (q a) (L1 x B)
  {
    double ub[3] = {0., 0., 0.}, r[3], rb[3];
    crossVjp(s.u2, B, Lb[1], ub, Bb);
    for (int i = 0; i < 3; ++i) {
      db[i] += ub[i];
      ab += ub[i] * s.k1[i];
      kb1[i] += a * ub[i];
    }
    cross(X.L[0], B, r);
    const double sc = q * a;
    const double scb = dot(Lb[1], r);
    qb += scb * a;
    ab += scb * q;
    for (int i = 0; i < 3; ++i) rb[i] = sc * Lb[1][i];
    crossVjp(X.L[0], B, rb, Lb[0], Bb);
  }
  // L1 = d x B
  crossVjp(d, B, Lb[0], db, Bb);
  // T4 = next(T3, h), T3 = next(T2, a), T2 = next(T1, a)
  tNextVjp(X.T[2], h, q, B, Tb[3], Tb[2], hb, qb, Bb);
  tNextVjp(X.T[1], a, q, B, Tb[2], Tb[1], ab, qb, Bb);
  tNextVjp(X.T[0], a, q, B, Tb[1], Tb[0], ab, qb, Bb);
  // T1
  const double(&t)[3][3] = Tb[0];
  qb += t[0][1] * B[2] - t[0][2] * B[1] - t[1][0] * B[2] + t[1][2] * B[0] + t[2][0] * B[1] -
        t[2][1] * B[0];
  Bb[0] += q * (t[1][2] - t[2][1]);
  Bb[1] += q * (t[2][0] - t[0][2]);
  Bb[2] += q * (t[0][1] - t[1][0]);
  hb += 0.5 * ab;
}

KF_HD void jtApply(const DMat &D, const JT &J, JT &O) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      O.A[i][j] = J.A[i][j] + D.DA[i][0] * J.B[0][j] + D.DA[i][1] * J.B[1][j] + D.DA[i][2] * J.B[2][j];
      O.B[i][j] = D.DB[i][0] * J.B[0][j] + D.DB[i][1] * J.B[1][j] + D.DB[i][2] * J.B[2][j];
    }
    O.a[i] = J.a[i] + D.DA[i][0] * J.c[0] + D.DA[i][1] * J.c[1] + D.DA[i][2] * J.c[2] + D.Da[i];
    O.c[i] = D.DB[i][0] * J.c[0] + D.DB[i][1] * J.c[1] + D.DB[i][2] * J.c[2] + D.Dc[i];
  }
  O.b = J.b + D.D37;
}

// Ob: adjoint of the output (consumed read-only); adds into Db and Jb
KF_HD void jtApplyVjp(const DMat &D, const JT &J, const JT &Ob, DMat &Db, JT &Jb) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      Jb.A[i][j] += Ob.A[i][j];
      for (int k = 0; k < 3; ++k) {
        Db.DA[i][k] += Ob.A[i][j] * J.B[k][j];
        Jb.B[k][j] += D.DA[i][k] * Ob.A[i][j];
        Db.DB[i][k] += Ob.B[i][j] * J.B[k][j];
        Jb.B[k][j] += D.DB[i][k] * Ob.B[i][j];
      }
    }
    Jb.a[i] += Ob.a[i];
    Db.Da[i] += Ob.a[i];
    Db.Dc[i] += Ob.c[i];
    for (int k = 0; k < 3; ++k) {
      Db.DA[i][k] += Ob.a[i] * J.c[k];
      Jb.c[k] += D.DA[i][k] * Ob.a[i];
      Db.DB[i][k] += Ob.c[i] * J.c[k];
      Jb.c[k] += D.DB[i][k] * Ob.c[i];
    }
  }
  Jb.b += Ob.b;
  Db.D37 += Ob.b;
}

// ---------------------------------------------------------------------------
// The RK4 step in a uniform field, evaluated through A v = v x B.  A^3 =
// -|B|^2 A, so every stage is a combination of c = d x B and e = c x B:
//   k1 = q c, k2 = q c + (h q^2/2) e, k3 = q(1 - x/4) c + (h q^2/2) e,
//   k4 = q(1 - x/2) c + h q^2 (1 - x/4) e,        x = h^2 q^2 |B|^2,
// and so is the step's transport matrix (T_n are the same polynomials in A):
//   pos' = pos + h d + h^2/6 (P c + Q e),   P = q(3 - x/4),  Q = h q^2
//   w = d + h/6 (Pd c + Qd e), d' = w/|w|,  Pd = q(6 - x),   Qd = h q^2 (3 - x/4)
//   err = h^2 |k1 - k2 - k3 + k4|_1 = h^2 |q| x/4 |c + h q e|_1
//   DA = h I + h^2/6 (P A + Q A^2),  DB = I + h/6 (Pd A + Qd A^2)
//   Da = h^2/6 ((3 - 3x/4) c + 2 h q e),  Dc = h/6 ((6 - 3x) c + h q (6 - x) e)
// (Da, Dc: the q-derivatives of the stage sums).  Algebraically identical to
// the stage-by-stage evaluation (EigenStepper.ipp:243-269 and :50-124), without
// its cancellation in k1 - k2 - k3 + k4, and about a third of its operations.
// ---------------------------------------------------------------------------
struct PolyStep {
  double c[3], e[3], beta, hq, x, P, Q, Pd, Qd;
  double v[3], F, S; // error estimate: err0 = F S, F = h^2 |q| x/4, S = |c + hq e|_1
  double err;
};

// c, e, |B|^2: fixed over the trials of one step
KF_HD void polyPrep(const double d[3], const double B[3], PolyStep &w) {
  cross(d, B, w.c);
  cross(w.c, B, w.e);
  w.beta = dot(B, B);
}
// coefficients and error estimate of a trial with step h
KF_HD void polyCoef(double q, double h, PolyStep &w) {
  w.hq = h * q;
  w.x = w.hq * w.hq * w.beta;
  w.P = q * (3. - 0.25 * w.x);
  w.Q = h * q * q;
  w.Pd = q * (6. - w.x);
  w.Qd = h * q * q * (3. - 0.25 * w.x);
  w.S = 0.;
  for (int i = 0; i < 3; ++i) {
    w.v[i] = w.c[i] + w.hq * w.e[i];
    w.S += fabs(w.v[i]);
  }
  w.F = h * h * fabs(q) * w.x * 0.25;
  const double e0 = w.F * w.S;
  w.err = e0 < 1e-20 ? 1e-20 : e0;
}
// err of a trial step (the accepted step adds polyAcceptFwd)
KF_HD void polyTrialFwd(const double d[3], double q, double h, const double B[3], PolyStep &w) {
  polyPrep(d, B, w);
  polyCoef(q, h, w);
}

struct PolyOut {
  double pos[3], dir[3], t, k4[3], w[3], n, in; // in = 1 / n
  DMat D;
};
// A = the matrix of v -> v x B, A2 = A^2 = B B^T - |B|^2 I
KF_HD void crossMatrix(const double B[3], double A[3][3], double A2[3][3], double beta) {
  A[0][0] = 0.;
  A[0][1] = B[2];
  A[0][2] = -B[1];
  A[1][0] = -B[2];
  A[1][1] = 0.;
  A[1][2] = B[0];
  A[2][0] = B[1];
  A[2][1] = -B[0];
  A[2][2] = 0.;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A2[i][j] = B[i] * B[j] - ((i == j) ? beta : 0.);
}

// fastNorm (the adjoint's reverse sweep, where the step is recomputed only
// for its derivatives): 1/|w| from rsqrt instead of a square root and a
// division; the fit's step keeps the latter
KF_HD void polyAcceptFwd(const double pos[3], const double d[3], double t, double q, double h,
                         double dtds, double d37, const double B[3], const PolyStep &w,
                         PolyOut &o, bool fastNorm = false) {
  // constants as products (a division by a literal is a full FP64 division)
  const double h6 = h * (1. / 6.), hh6 = h * h6;
  for (int i = 0; i < 3; ++i) {
    o.pos[i] = pos[i] + (h * d[i] + hh6 * (w.P * w.c[i] + w.Q * w.e[i]));
    o.w[i] = d[i] + h6 * (w.Pd * w.c[i] + w.Qd * w.e[i]);
  }
  if (fastNorm) {
    const double n2 = dot(o.w, o.w);
    o.in = rsqrtD(n2);
    o.n = n2 * o.in;
  } else {
    o.n = sqrt(dot(o.w, o.w));
    o.in = 1. / o.n;
  }
  for (int i = 0; i < 3; ++i) o.dir[i] = o.w[i] * o.in;
  o.t = t + h * dtds;
  const double a4 = q * (1. - 0.5 * w.x), b4 = h * q * q * (1. - 0.25 * w.x);
  for (int i = 0; i < 3; ++i) o.k4[i] = a4 * w.c[i] + b4 * w.e[i];
  double A[3][3], A2[3][3];
  crossMatrix(B, A, A2, w.beta);
  const double ca = hh6 * w.P, cb = hh6 * w.Q, cc = h6 * w.Pd, cd = h6 * w.Qd;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      o.D.DA[i][j] = ((i == j) ? h : 0.) + (ca * A[i][j] + cb * A2[i][j]);
      o.D.DB[i][j] = ((i == j) ? 1. : 0.) + (cc * A[i][j] + cd * A2[i][j]);
    }
  const double ea = 3. - 0.75 * w.x, eb = 2. * w.hq;
  const double fa = 6. - 3. * w.x, fb = w.hq * (6. - w.x);
  for (int i = 0; i < 3; ++i) {
    o.D.Da[i] = hh6 * (ea * w.c[i] + eb * w.e[i]);
    o.D.Dc[i] = h6 * (fa * w.c[i] + fb * w.e[i]);
  }
  o.D.D37 = h * d37;
}

// <G, A> and <G, A2> and their B-gradients (scaled by s)
KF_HD double fro(const double G[3][3], const double M[3][3]) {
  double r = 0.;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r += G[i][j] * M[i][j];
  return r;
}
KF_HD void froAVjp(const double G[3][3], double s, double Bb[3]) {
  Bb[0] += s * (G[1][2] - G[2][1]);
  Bb[1] += s * (G[2][0] - G[0][2]);
  Bb[2] += s * (G[0][1] - G[1][0]);
}
KF_HD void froA2Vjp(const double G[3][3], const double B[3], double s, double Bb[3]) {
  const double tr = G[0][0] + G[1][1] + G[2][2];
  for (int i = 0; i < 3; ++i) {
    double g = 0.;
    for (int j = 0; j < 3; ++j) g += (G[i][j] + G[j][i]) * B[j];
    Bb[i] += s * (g - 2. * tr * B[i]);
  }
}

// adjoint of the trial's error estimate: errb -> d, q, h, B
KF_HD void polyErrVjp(const double d[3], double q, double h, const double B[3], const PolyStep &w,
                      double errb, double db[3], double &qb, double &hb, double Bb[3]) {
  if (errb == 0. || w.F * w.S <= 1e-20) return;
  const double Sb = errb * w.F, Fb = errb * w.S;
  double cb[3], eb[3], hqb = 0.;
  for (int i = 0; i < 3; ++i) {
    const double vb = Sb * (w.v[i] > 0. ? 1. : (w.v[i] < 0. ? -1. : 0.));
    cb[i] = vb;
    eb[i] = w.hq * vb;
    hqb += vb * w.e[i];
  }
  // F = h^2 |q| x / 4
  hb += Fb * 2. * w.F / h;
  qb += Fb * w.F / q;
  const double xb = Fb * h * h * fabs(q) * 0.25;
  hqb += xb * 2. * w.hq * w.beta;
  const double betab = xb * w.hq * w.hq;
  hb += hqb * q;
  qb += hqb * h;
  for (int i = 0; i < 3; ++i) Bb[i] += 2. * betab * B[i];
  crossVjp(w.c, B, eb, cb, Bb);
  crossVjp(d, B, cb, db, Bb);
}

// adjoint of the accepted step: (pos', dir', t', k4, D) -> pos, d, t, q, h, dtds, d37, B
KF_HD void polyAcceptVjp(const double d[3], double q, double h, double dtds, double d37,
                         const double B[3], const PolyStep &w, const PolyOut &o,
                         const double posb_[3], const double dirb_[3], double tb_,
                         const double k4b[3], const DMat &Db, double posb[3], double db[3],
                         double &tb, double &qb, double &hb, double &dtdsb, double &d37b,
                         double Bb[3]) {
  const double h6 = h * (1. / 6.), hh6 = h * h6, h3 = h * (1. / 3.), k6 = 1. / 6.;
  double cb[3] = {0., 0., 0.}, eb[3] = {0., 0., 0.};
  double Pb = 0., Qb = 0., Pdb = 0., Qdb = 0., xb = 0., hqb = 0.;
  // time and D37
  tb += tb_;
  hb += tb_ * dtds + Db.D37 * d37;
  dtdsb += tb_ * h;
  d37b += Db.D37 * h;
  // Da = hh6 (ea c + eb e), Dc = h6 (fa c + fb e)
  {
    const double ea = 3. - 0.75 * w.x, ebb = 2. * w.hq;
    const double fa = 6. - 3. * w.x, fbb = w.hq * (6. - w.x);
    double gc = 0., ge = 0., hc = 0., he = 0.;
    for (int i = 0; i < 3; ++i) {
      cb[i] += hh6 * ea * Db.Da[i] + h6 * fa * Db.Dc[i];
      eb[i] += hh6 * ebb * Db.Da[i] + h6 * fbb * Db.Dc[i];
      gc += Db.Da[i] * w.c[i];
      ge += Db.Da[i] * w.e[i];
      hc += Db.Dc[i] * w.c[i];
      he += Db.Dc[i] * w.e[i];
    }
    hb += h3 * (ea * gc + ebb * ge) + (fa * hc + fbb * he) * k6;
    xb += hh6 * (-0.75) * gc + h6 * (-3.) * hc + h6 * (-w.hq) * he;
    hqb += hh6 * 2. * ge + h6 * (6. - w.x) * he;
  }
  // DA = h I + hh6 (P A + Q A2), DB = I + h6 (Pd A + Qd A2)
  {
    double A[3][3], A2[3][3];
    crossMatrix(B, A, A2, w.beta);
    const double gA = fro(Db.DA, A), gA2 = fro(Db.DA, A2);
    const double fA = fro(Db.DB, A), fA2 = fro(Db.DB, A2);
    hb += Db.DA[0][0] + Db.DA[1][1] + Db.DA[2][2];
    hb += h3 * (w.P * gA + w.Q * gA2) + (w.Pd * fA + w.Qd * fA2) * k6;
    Pb += hh6 * gA;
    Qb += hh6 * gA2;
    Pdb += h6 * fA;
    Qdb += h6 * fA2;
    froAVjp(Db.DA, hh6 * w.P, Bb);
    froA2Vjp(Db.DA, B, hh6 * w.Q, Bb);
    froAVjp(Db.DB, h6 * w.Pd, Bb);
    froA2Vjp(Db.DB, B, h6 * w.Qd, Bb);
  }
  // k4 = a4 c + b4 e
  {
    const double a4 = q * (1. - 0.5 * w.x), b4 = h * q * q * (1. - 0.25 * w.x);
    double a4b = 0., b4b = 0.;
    for (int i = 0; i < 3; ++i) {
      cb[i] += a4 * k4b[i];
      eb[i] += b4 * k4b[i];
      a4b += k4b[i] * w.c[i];
      b4b += k4b[i] * w.e[i];
    }
    qb += a4b * (1. - 0.5 * w.x) + b4b * 2. * h * q * (1. - 0.25 * w.x);
    xb += -a4b * 0.5 * q - b4b * 0.25 * h * q * q;
    hb += b4b * q * q * (1. - 0.25 * w.x);
  }
  // pos' = pos + h d + hh6 (P c + Q e)
  {
    double pc = 0., pe = 0., pd = 0.;
    for (int i = 0; i < 3; ++i) {
      posb[i] += posb_[i];
      db[i] += h * posb_[i];
      cb[i] += hh6 * w.P * posb_[i];
      eb[i] += hh6 * w.Q * posb_[i];
      pc += posb_[i] * w.c[i];
      pe += posb_[i] * w.e[i];
      pd += posb_[i] * d[i];
    }
    hb += pd + h3 * (w.P * pc + w.Q * pe);
    Pb += hh6 * pc;
    Qb += hh6 * pe;
  }
  // d' = w/n, w = d + h6 (Pd c + Qd e)
  {
    const double pr = dot(o.dir, dirb_);
    double wb[3], wc = 0., we = 0.;
    for (int i = 0; i < 3; ++i) {
      wb[i] = (dirb_[i] - o.dir[i] * pr) * o.in;
      db[i] += wb[i];
      cb[i] += h6 * w.Pd * wb[i];
      eb[i] += h6 * w.Qd * wb[i];
      wc += wb[i] * w.c[i];
      we += wb[i] * w.e[i];
    }
    hb += (w.Pd * wc + w.Qd * we) * k6;
    Pdb += h6 * wc;
    Qdb += h6 * we;
  }
  // scalar coefficients
  qb += Pb * (3. - 0.25 * w.x) + Qb * 2. * h * q + Pdb * (6. - w.x) +
        Qdb * 2. * h * q * (3. - 0.25 * w.x);
  hb += Qb * q * q + Qdb * q * q * (3. - 0.25 * w.x);
  xb += -Pb * 0.25 * q - Pdb * q - Qdb * 0.25 * h * q * q;
  hqb += xb * 2. * w.hq * w.beta;
  const double betab = xb * w.hq * w.hq;
  hb += hqb * q;
  qb += hqb * h;
  for (int i = 0; i < 3; ++i) Bb[i] += 2. * betab * B[i];
  crossVjp(w.c, B, eb, cb, Bb);
  crossVjp(d, B, cb, db, Bb);
}

// ---------------------------------------------------------------------------
// Straight-line distance to a plane along d (SteppingHelper.hpp:31-65 with
// PlanarHelper::intersectionEstimate): path = T.(c - pos) / (T.d)
// ---------------------------------------------------------------------------
KF_HD double pathFwd(const double pos[3], const double d[3], const double c[3],
                     const double T[3]) {
  return (T[0] * (c[0] - pos[0]) + T[1] * (c[1] - pos[1]) + T[2] * (c[2] - pos[2])) / dot(d, T);
}
KF_HD void pathVjp(const double pos[3], const double d[3], const double c[3], const double T[3],
                   double pb, double posb[3], double db[3], double cb[3], double Tb[3]) {
  const double iden = 1. / dot(d, T);
  const double path = (T[0] * (c[0] - pos[0]) + T[1] * (c[1] - pos[1]) + T[2] * (c[2] - pos[2])) *
                      iden;
  const double g = pb * iden;
  for (int i = 0; i < 3; ++i) {
    posb[i] -= T[i] * g;
    cb[i] += T[i] * g;
    db[i] -= path * T[i] * g;
    Tb[i] += ((c[i] - pos[i]) - path * d[i]) * g;
  }
}

// Step-size scale after a rejected trial (EigenStepper.ipp:281-290):
// clamp(pow(tol / |2 err|, 1/4), 0.25, 4); dscale/derr in *dsde
KF_HD double accScale(double err, double tol, double *dsde) {
  const double raw = pow(tol / fabs(2. * err), 0.25);
  if (raw <= 0.25) {
    *dsde = 0.;
    return 0.25;
  }
  if (raw >= 4.) {
    *dsde = 0.;
    return 4.;
  }
  *dsde = -0.25 * raw / err;
  return raw;
}

// ---------------------------------------------------------------------------
// Bound state on a plane with covariance transport and re-initialisation
// (EigenStepper.ipp:516-540, CovarianceEngine.hpp:106-125,169-201,269-290,
// PlaneSurface.ipp:122-204):
//   Pt, Dd, R3 = rows of jacTransport * jacToGlobal (position, direction,
//   time) on columns 0..4; sVec = T.Pt / T.d; the derivative (d, dt/ds, k4 of
//   the last step, zero right after a reset) times sVec is subtracted; J =
//   jacToLocal * that; C' = J C J^T; the stored Jacobian is J rows 0-3,5 x
//   cols 0-4; the new jacToGlobal is built from d and the plane axes.
// ---------------------------------------------------------------------------
struct Frame {
  double c[3], U[3], V[3], T[3];
};
struct FrameBar {
  double c[3], U[3], V[3], T[3];
};
struct Gj {
  double g03[3][4], g46[3][2];
};

KF_HD int ut6(int i, int j) { return i * 6 - (i * (i - 1)) / 2 + (j - i); }
KF_HD int si6(int i, int j) { return i <= j ? ut6(i, j) : ut6(j, i); }

// direction-dependent coefficients (jacToLocal rows 2-3 and jacToGlobal rows 4-6)
struct DirCoef {
  double j24, j25, j34, j35, j36;
  double g46[3][2];
};
KF_HD void dirCoefFwd(const double d[3], DirCoef &k) {
  const double x = d[0], y = d[1], z = d[2];
  const double r2 = x * x + y * y, invS = rsqrtD(r2);
  const double cosT = z, sinT = r2 * invS;
  const double cosP = x * invS, sinP = y * invS;
  k.j24 = -sinP * invS;
  k.j25 = cosP * invS;
  k.j34 = cosP * cosT;
  k.j35 = sinP * cosT;
  k.j36 = -sinT;
  k.g46[0][0] = (-sinT) * sinP;
  k.g46[0][1] = cosT * cosP;
  k.g46[1][0] = sinT * cosP;
  k.g46[1][1] = cosT * sinP;
  k.g46[2][0] = 0.;
  k.g46[2][1] = -sinT;
}
KF_HD void dirCoefVjp(const double d[3], const DirCoef &kb, double db[3]) {
  const double x = d[0], y = d[1], z = d[2];
  // powers of 1/s, s = sqrt(x^2 + y^2), from one reciprocal square root
  const double is = rsqrtD(x * x + y * y), ir2 = is * is, is3 = ir2 * is, ir4 = ir2 * ir2;
  // j24 = -y / r2, j25 = x / r2
  db[0] += kb.j24 * (2. * x * y * ir4) + kb.j25 * ((y * y - x * x) * ir4);
  db[1] += kb.j24 * ((y * y - x * x) * ir4) + kb.j25 * (-2. * x * y * ir4);
  // j34 = x z / s, j35 = y z / s, j36 = -s
  db[0] += kb.j34 * (z * y * y * is3) + kb.j35 * (-x * y * z * is3) + kb.j36 * (-x * is);
  db[1] += kb.j34 * (-x * y * z * is3) + kb.j35 * (z * x * x * is3) + kb.j36 * (-y * is);
  db[2] += kb.j34 * (x * is) + kb.j35 * (y * is);
  // g46: [[-y, x z / s], [x, y z / s], [0, -s]]
  db[1] -= kb.g46[0][0];
  db[0] += kb.g46[1][0];
  db[0] += kb.g46[0][1] * (z * y * y * is3) + kb.g46[1][1] * (-x * y * z * is3) +
           kb.g46[2][1] * (-x * is);
  db[1] += kb.g46[0][1] * (-x * y * z * is3) + kb.g46[1][1] * (z * x * x * is3) +
           kb.g46[2][1] * (-y * is);
  db[2] += kb.g46[0][1] * (x * is) + kb.g46[1][1] * (y * is);
}

struct BoundIn {
  double pos[3], dir[3], q, p, t;
  JT J;
  Gj G;
  bool stepped;
  double dtds, k4[3];
  double C[21];
};
struct BoundOut {
  double pred[6], Cp[21], Jst[25];
  Gj G; // new jacToGlobal
};
struct BoundTmp {
  double Pt0[3][5], Dd0[3][5], R30[5]; // before the derivative subtraction
  double Pt[3][5], Dd[3][5], R3[5];
  double sVec[5], nv[3], dp, idp, der[7];
  double Jf[6][6], M[6][6];
  DirCoef k;
};

// full = false: the reverse sweep's recomputation; the predicted parameters
// come from the stored state and only covariance rows 0-1 (all the gain and
// its adjoint read) are formed
KF_HD void boundFwd(const BoundIn &in, const Frame &f, BoundOut &o, BoundTmp &w,
                    bool full = true) {
  for (int r = 0; r < 3; ++r) {
    w.Pt0[r][0] = in.G.g03[r][0];
    w.Pt0[r][1] = in.G.g03[r][1];
    for (int c = 0; c < 2; ++c) {
      w.Pt0[r][2 + c] = in.G.g03[r][2 + c] + in.J.A[r][0] * in.G.g46[0][c] +
                        in.J.A[r][1] * in.G.g46[1][c] + in.J.A[r][2] * in.G.g46[2][c];
      w.Dd0[r][2 + c] = in.J.B[r][0] * in.G.g46[0][c] + in.J.B[r][1] * in.G.g46[1][c] +
                        in.J.B[r][2] * in.G.g46[2][c];
    }
    w.Pt0[r][4] = in.J.a[r];
    w.Dd0[r][0] = 0.;
    w.Dd0[r][1] = 0.;
    w.Dd0[r][4] = in.J.c[r];
  }
  for (int c = 0; c < 4; ++c) w.R30[c] = 0.;
  w.R30[4] = in.J.b;
  w.dp = dot(f.T, in.dir);
  w.idp = 1. / w.dp;
  for (int i = 0; i < 3; ++i) w.nv[i] = f.T[i] * w.idp;
  for (int c = 0; c < 5; ++c)
    w.sVec[c] = w.nv[0] * w.Pt0[0][c] + w.nv[1] * w.Pt0[1][c] + w.nv[2] * w.Pt0[2][c];
  for (int r = 0; r < 3; ++r) {
    w.der[r] = in.stepped ? in.dir[r] : 0.;
    w.der[4 + r] = in.stepped ? in.k4[r] : 0.;
  }
  w.der[3] = in.stepped ? in.dtds : 0.;
  for (int c = 0; c < 5; ++c) {
    for (int r = 0; r < 3; ++r) {
      w.Pt[r][c] = w.Pt0[r][c] - w.der[r] * w.sVec[c];
      w.Dd[r][c] = w.Dd0[r][c] - w.der[4 + r] * w.sVec[c];
    }
    w.R3[c] = w.R30[c] - w.der[3] * w.sVec[c];
  }
  dirCoefFwd(in.dir, w.k);
  double(&J)[6][6] = w.Jf;
  for (int c = 0; c < 5; ++c) {
    J[0][c] = f.U[0] * w.Pt[0][c] + f.U[1] * w.Pt[1][c] + f.U[2] * w.Pt[2][c];
    J[1][c] = f.V[0] * w.Pt[0][c] + f.V[1] * w.Pt[1][c] + f.V[2] * w.Pt[2][c];
    J[2][c] = w.k.j24 * w.Dd[0][c] + w.k.j25 * w.Dd[1][c];
    J[3][c] = w.k.j34 * w.Dd[0][c] + w.k.j35 * w.Dd[1][c] + w.k.j36 * w.Dd[2][c];
    J[4][c] = (c == 4) ? 1. : 0.;
    J[5][c] = w.R3[c];
  }
  for (int r = 0; r < 6; ++r) J[r][5] = (r == 5) ? 1. : 0.;
  // M = J C and C' = M J^T on the structure: row 4 of J is e4, column 5 is e5
  // (the recomputation needs rows 0-1 only; the VJP does not read M)
  for (int i = 0; i < (full ? 6 : 2); ++i)
    for (int j = 0; j < 6; ++j) {
      if (i == 4) {
        w.M[4][j] = in.C[si6(4, j)];
        continue;
      }
      double s = 0.;
      for (int k = 0; k < 5; ++k) s += J[i][k] * in.C[si6(k, j)];
      if (i == 5) s += in.C[si6(5, j)];
      w.M[i][j] = s;
    }
  for (int i = 0; i < (full ? 6 : 2); ++i)
    for (int j = i; j < 6; ++j) {
      double s;
      if (j == 4) {
        s = w.M[i][4];
      } else {
        s = 0.;
        for (int k = 0; k < 5; ++k) s += w.M[i][k] * J[j][k];
        if (j == 5) s += w.M[i][5];
      }
      o.Cp[ut6(i, j)] = s;
    }
  for (int c = 0; c < 5; ++c) {
    o.Jst[c] = J[0][c];
    o.Jst[5 + c] = J[1][c];
    o.Jst[10 + c] = J[2][c];
    o.Jst[15 + c] = J[3][c];
    o.Jst[20 + c] = J[5][c];
  }
  for (int r = 0; r < 3; ++r) {
    o.G.g03[r][0] = f.U[r];
    o.G.g03[r][1] = f.V[r];
    o.G.g03[r][2] = 0.;
    o.G.g03[r][3] = 0.;
    o.G.g46[r][0] = w.k.g46[r][0];
    o.G.g46[r][1] = w.k.g46[r][1];
  }
  if (!full) return;
  double dd[3];
  for (int i = 0; i < 3; ++i) dd[i] = in.pos[i] - f.c[i];
  o.pred[0] = dot(f.U, dd);
  o.pred[1] = dot(f.V, dd);
  // angles from the direction, q/p as the stepper holds it (the fit's
  // boundAngles)
  const double pt = sqrt(in.dir[0] * in.dir[0] + in.dir[1] * in.dir[1]);
  o.pred[2] = atan2(in.dir[1], in.dir[0]);
  o.pred[3] = atan2(pt, in.dir[2]);
  o.pred[4] = in.q / in.p;
  o.pred[5] = in.t;
}

struct BoundInBar {
  double pos[3], dir[3], p, t;
  JT J;
  Gj G;
  double dtds, k4[3];
  double C[21];
};
KF_HD void boundInBarZero(BoundInBar &b) {
  for (int i = 0; i < 3; ++i) b.pos[i] = b.dir[i] = b.k4[i] = 0.;
  b.p = b.t = b.dtds = 0.;
  jtZero(b.J);
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) b.G.g03[r][c] = 0.;
    b.G.g46[r][0] = b.G.g46[r][1] = 0.;
  }
  for (int e = 0; e < 21; ++e) b.C[e] = 0.;
}
KF_HD void frameBarZero(FrameBar &b) {
  for (int i = 0; i < 3; ++i) b.c[i] = b.U[i] = b.V[i] = b.T[i] = 0.;
}

// ob: adjoints of pred, Cp, Jst and the new G; adds into ib and fb
KF_HD void boundVjp(const BoundIn &in, const Frame &f, const BoundOut &o, const BoundTmp &w,
                    const BoundOut &ob, BoundInBar &ib, FrameBar &fb) {
  // ---- bound parameters
  double dd[3];
  for (int i = 0; i < 3; ++i) dd[i] = in.pos[i] - f.c[i];
  for (int i = 0; i < 3; ++i) {
    fb.U[i] += ob.pred[0] * dd[i];
    fb.V[i] += ob.pred[1] * dd[i];
    const double g = ob.pred[0] * f.U[i] + ob.pred[1] * f.V[i];
    ib.pos[i] += g;
    fb.c[i] -= g;
  }
  {
    const double x = in.dir[0], y = in.dir[1], z = in.dir[2];
    const double r2 = x * x + y * y, rho2 = r2 + z * z;
    const double is = rsqrtD(r2), s = r2 * is, ir2 = is * is, irho2 = 1. / rho2;
    // phi = atan2(y, x), theta = atan2(s, z) (scale-free in the momentum)
    ib.dir[0] += ob.pred[2] * (-y * ir2);
    ib.dir[1] += ob.pred[2] * (x * ir2);
    const double sb = ob.pred[3] * (z * irho2);
    ib.dir[2] += ob.pred[3] * (-s * irho2);
    ib.dir[0] += sb * x * is;
    ib.dir[1] += sb * y * is;
    // q/p = q / p: d(q/p)/dp = -q / p^2 = -q (q/p)^2 (q = +-1)
    ib.p += ob.pred[4] * (-in.q * o.pred[4] * o.pred[4]);
  }
  ib.t += ob.pred[5];
  // ---- new jacToGlobal
  DirCoef kb;
  kb.j24 = kb.j25 = kb.j34 = kb.j35 = kb.j36 = 0.;
  for (int r = 0; r < 3; ++r) {
    fb.U[r] += ob.G.g03[r][0];
    fb.V[r] += ob.G.g03[r][1];
    kb.g46[r][0] = ob.G.g46[r][0];
    kb.g46[r][1] = ob.G.g46[r][1];
  }
  // ---- C' = J C J^T and the stored Jacobian (J: row 4 = e4, column 5 = e5).
  // W is the upper-triangle adjoint of C' and Ws = W + W^T; with X = Ws J,
  //   J-bar = Ws J C = X C on the free entries (rows 0-3, 5; columns 0-4),
  //   C-bar on the stored triangle = (J^T X)_kl for k < l, (J^T X)_kk / 2
  // (J^T Ws J is the full-matrix gradient plus its transpose)
  double Ws[6][6], Jb[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      Ws[i][j] = (i == j) ? 2. * ob.Cp[ut6(i, i)] : ob.Cp[ut6(i < j ? i : j, i < j ? j : i)];
      Jb[i][j] = 0.;
    }
  const double(&J)[6][6] = w.Jf;
  constexpr int kFree[5] = {0, 1, 2, 3, 5}; // J's rows off e4
  double X[6][6];
  for (int a = 0; a < 6; ++a) {
    for (int k = 0; k < 5; ++k) {
      double s = (k == 4) ? Ws[a][4] : 0.;
      for (int ii = 0; ii < 5; ++ii) s += Ws[a][kFree[ii]] * J[kFree[ii]][k];
      X[a][k] = s;
    }
    X[a][5] = Ws[a][5];
  }
  for (int ai = 0; ai < 5; ++ai) {
    const int a = kFree[ai];
    for (int b = 0; b < 5; ++b) {
      double s = 0.;
      for (int k = 0; k < 6; ++k) s += X[a][k] * in.C[si6(k, b)];
      Jb[a][b] += s;
    }
  }
  for (int k = 0; k < 6; ++k)
    for (int l = k; l < 6; ++l) {
      double s;
      if (k == 5) {
        s = X[5][l];
      } else {
        s = (k == 4) ? X[4][l] : 0.;
        for (int ii = 0; ii < 5; ++ii) s += J[kFree[ii]][k] * X[kFree[ii]][l];
      }
      ib.C[ut6(k, l)] += (k == l) ? 0.5 * s : s;
    }
  for (int c = 0; c < 5; ++c) {
    Jb[0][c] += ob.Jst[c];
    Jb[1][c] += ob.Jst[5 + c];
    Jb[2][c] += ob.Jst[10 + c];
    Jb[3][c] += ob.Jst[15 + c];
    Jb[5][c] += ob.Jst[20 + c];
  }
  // ---- J rows from Pt, Dd, R3 and the direction coefficients
  double Ptb[3][5], Ddb[3][5], R3b[5];
  for (int c = 0; c < 5; ++c) {
    for (int r = 0; r < 3; ++r) {
      fb.U[r] += Jb[0][c] * w.Pt[r][c];
      fb.V[r] += Jb[1][c] * w.Pt[r][c];
      Ptb[r][c] = Jb[0][c] * f.U[r] + Jb[1][c] * f.V[r];
    }
    kb.j24 += Jb[2][c] * w.Dd[0][c];
    kb.j25 += Jb[2][c] * w.Dd[1][c];
    kb.j34 += Jb[3][c] * w.Dd[0][c];
    kb.j35 += Jb[3][c] * w.Dd[1][c];
    kb.j36 += Jb[3][c] * w.Dd[2][c];
    Ddb[0][c] = w.k.j24 * Jb[2][c] + w.k.j34 * Jb[3][c];
    Ddb[1][c] = w.k.j25 * Jb[2][c] + w.k.j35 * Jb[3][c];
    Ddb[2][c] = w.k.j36 * Jb[3][c];
    R3b[c] = Jb[5][c];
  }
  dirCoefVjp(in.dir, kb, ib.dir);
  // ---- derivative subtraction: X = X0 - der (x) sVec
  double sVb[5] = {0., 0., 0., 0., 0.}, derb[7] = {0., 0., 0., 0., 0., 0., 0.};
  for (int c = 0; c < 5; ++c) {
    for (int r = 0; r < 3; ++r) {
      derb[r] -= Ptb[r][c] * w.sVec[c];
      derb[4 + r] -= Ddb[r][c] * w.sVec[c];
      sVb[c] -= Ptb[r][c] * w.der[r] + Ddb[r][c] * w.der[4 + r];
    }
    derb[3] -= R3b[c] * w.sVec[c];
    sVb[c] -= R3b[c] * w.der[3];
  }
  if (in.stepped) {
    for (int r = 0; r < 3; ++r) {
      ib.dir[r] += derb[r];
      ib.k4[r] += derb[4 + r];
    }
    ib.dtds += derb[3];
  }
  // ---- sVec = nv . Pt0, nv = T / (T.d)
  double nvb[3] = {0., 0., 0.};
  for (int c = 0; c < 5; ++c)
    for (int r = 0; r < 3; ++r) {
      nvb[r] += sVb[c] * w.Pt0[r][c];
      Ptb[r][c] += sVb[c] * w.nv[r];
    }
  {
    const double dpb = -dot(nvb, f.T) * (w.idp * w.idp);
    for (int i = 0; i < 3; ++i) {
      fb.T[i] += nvb[i] * w.idp + dpb * in.dir[i];
      ib.dir[i] += dpb * f.T[i];
    }
  }
  // ---- applyTransport
  for (int r = 0; r < 3; ++r) {
    ib.G.g03[r][0] += Ptb[r][0];
    ib.G.g03[r][1] += Ptb[r][1];
    for (int c = 0; c < 2; ++c) {
      ib.G.g03[r][2 + c] += Ptb[r][2 + c];
      for (int m = 0; m < 3; ++m) {
        ib.J.A[r][m] += Ptb[r][2 + c] * in.G.g46[m][c];
        ib.G.g46[m][c] += Ptb[r][2 + c] * in.J.A[r][m] + Ddb[r][2 + c] * in.J.B[r][m];
        ib.J.B[r][m] += Ddb[r][2 + c] * in.G.g46[m][c];
      }
    }
    ib.J.a[r] += Ptb[r][4];
    ib.J.c[r] += Ddb[r][4];
  }
  ib.J.b += R3b[4];
}

// ---------------------------------------------------------------------------
// Gain-matrix update (GainMatrixUpdater.hpp:34-106), H = [I2 0], FP64 form
//   S = H C H^T + V, K = C H^T S^-1, x_f = x_p + K (m - H x_p),
//   C_f = C - K H C (upper triangle)
// ---------------------------------------------------------------------------
struct FilterTmp {
  double i00, i01, i10, i11, r0, r1, K0[6], K1[6];
};
KF_HD void filterFwd(const double pred[6], const double C[21], const double mv[5],
                     double filt[6], double cf[21], double *chi2, FilterTmp &w) {
  const double S00 = C[0] + mv[2], S01 = C[1] + mv[3], S10 = C[1] + mv[3], S11 = C[6] + mv[4];
  const double idet = 1. / (S00 * S11 - S01 * S10);
  w.i00 = S11 * idet;
  w.i01 = -S01 * idet;
  w.i10 = -S10 * idet;
  w.i11 = S00 * idet;
  w.r0 = mv[0] - pred[0];
  w.r1 = mv[1] - pred[1];
  *chi2 = w.r0 * (w.i00 * w.r0 + w.i01 * w.r1) + w.r1 * (w.i10 * w.r0 + w.i11 * w.r1);
  for (int i = 0; i < 6; ++i) {
    const double c0 = C[si6(i, 0)], c1 = C[si6(i, 1)];
    w.K0[i] = c0 * w.i00 + c1 * w.i10;
    w.K1[i] = c0 * w.i01 + c1 * w.i11;
  }
  for (int i = 0; i < 6; ++i) filt[i] = pred[i] + (w.K0[i] * w.r0 + w.K1[i] * w.r1);
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j)
      cf[ut6(i, j)] = C[ut6(i, j)] - w.K0[i] * C[si6(0, j)] - w.K1[i] * C[si6(1, j)];
}
KF_HD void filterVjp(const double C[21], const FilterTmp &w, const double filtb[6],
                     const double cfb[21], double predb[6], double Cb[21]) {
  double K0b[6], K1b[6], r0b = 0., r1b = 0.;
  for (int i = 0; i < 6; ++i) K0b[i] = K1b[i] = 0.;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j) {
      const double g = cfb[ut6(i, j)];
      Cb[ut6(i, j)] += g;
      K0b[i] -= g * C[si6(0, j)];
      K1b[i] -= g * C[si6(1, j)];
      Cb[si6(0, j)] -= g * w.K0[i];
      Cb[si6(1, j)] -= g * w.K1[i];
    }
  for (int i = 0; i < 6; ++i) {
    predb[i] += filtb[i];
    K0b[i] += filtb[i] * w.r0;
    K1b[i] += filtb[i] * w.r1;
    r0b += filtb[i] * w.K0[i];
    r1b += filtb[i] * w.K1[i];
  }
  double i00b = 0., i01b = 0., i10b = 0., i11b = 0.;
  for (int i = 0; i < 6; ++i) {
    const double c0 = C[si6(i, 0)], c1 = C[si6(i, 1)];
    Cb[si6(i, 0)] += K0b[i] * w.i00 + K1b[i] * w.i01;
    Cb[si6(i, 1)] += K0b[i] * w.i10 + K1b[i] * w.i11;
    i00b += K0b[i] * c0;
    i10b += K0b[i] * c1;
    i01b += K1b[i] * c0;
    i11b += K1b[i] * c1;
  }
  predb[0] -= r0b;
  predb[1] -= r1b;
  // S-bar = -Si^T Ib Si^T
  const double a00 = w.i00 * i00b + w.i10 * i10b, a01 = w.i00 * i01b + w.i10 * i11b;
  const double a10 = w.i01 * i00b + w.i11 * i10b, a11 = w.i01 * i01b + w.i11 * i11b;
  const double S00b = -(a00 * w.i00 + a01 * w.i01), S01b = -(a00 * w.i10 + a01 * w.i11);
  const double S10b = -(a10 * w.i00 + a11 * w.i01), S11b = -(a10 * w.i10 + a11 * w.i11);
  Cb[0] += S00b;
  Cb[1] += S01b + S10b;
  Cb[6] += S11b;
}

// ---------------------------------------------------------------------------
// Stepper update from filtered plane parameters (EigenStepper.ipp:554-564,
// coordinate_transformations.hpp:145-158) and the per-leg constants
//   pos = c + U x0 + V x1, d = unit(cos x2 sin x3, sin x2 sin x3, cos x3),
//   p = |1/x4|, t = x5;  qop = q/p, dtds = sqrt(1 + (m/p)^2), d37 = m^2 q/(p dtds)
// ---------------------------------------------------------------------------
// the stepper update from the filtered angles' sines and cosines
// trig = (sin phi, cos phi, sin theta, cos theta)
KF_HD void updateFwdTrig(const Frame &f, const double x[6], const double trig[4], double pos[3],
                         double d[3], double *p, double *t) {
  for (int r = 0; r < 3; ++r) pos[r] = f.U[r] * x[0] + f.V[r] * x[1] + f.c[r];
  const double sp = trig[0], cp = trig[1], st = trig[2], ct = trig[3];
  const double v[3] = {cp * st, sp * st, ct};
  const double in = rsqrtD(dot(v, v));
  for (int i = 0; i < 3; ++i) d[i] = v[i] * in;
  *p = fabs(1. / x[4]);
  *t = x[5];
}
KF_HD void updateFwd(const Frame &f, const double x[6], double pos[3], double d[3], double *p,
                     double *t, double trig[4] = nullptr) {
  double tr[4];
  sinCos(x[2], tr[0], tr[1]);
  sinCos(x[3], tr[2], tr[3]);
  if (trig)
    for (int e = 0; e < 4; ++e) trig[e] = tr[e];
  updateFwdTrig(f, x, tr, pos, d, p, t);
}
// Sines and cosines of the filtered angles phi_p + dphi, theta_p + dth from
// the predicted unit direction d (cos phi_p = d0 / s, sin phi_p = d1 / s,
// cos theta_p = d2, sin theta_p = s = |(d0, d1)|) by angle addition, with
// Taylor series for the corrections (|delta| <= 0.02: truncation below
// 1e-20), as the fit's stepper update does; false for a larger correction
// or a direction within 1e-6 of the z axis
KF_HD bool trigByAddition(const double d[3], double dphi, double dth, double trig[4]) {
  const double s2 = d[0] * d[0] + d[1] * d[1];
  if (!(fabs(dphi) <= 0.02) || !(fabs(dth) <= 0.02) || !(s2 > 1e-12)) return false;
  auto sinCosSmall = [](double x, double &sn, double &cs) {
    const double x2 = x * x;
    sn = x + x * x2 * (-1. / 6. + x2 * (1. / 120. + x2 * (-1. / 5040.)));
    cs = 1. + x2 * (-0.5 + x2 * (1. / 24. + x2 * (-1. / 720. + x2 * (1. / 40320.))));
  };
  double sdp, cdp, sdt, cdt;
  sinCosSmall(dphi, sdp, cdp);
  sinCosSmall(dth, sdt, cdt);
  const double is = rsqrtD(s2), s = s2 * is;
  const double cp0 = d[0] * is, sp0 = d[1] * is;
  trig[0] = sp0 * cdp + cp0 * sdp;
  trig[1] = cp0 * cdp - sp0 * sdp;
  trig[2] = s * cdt + d[2] * sdt;
  trig[3] = d[2] * cdt - s * sdt;
  return true;
}
// sp, cp, st, ct: sin/cos of x[2] and x[3] (as evaluated by updateFwd)
KF_HD void updateVjp(const Frame &f, const double x[6], const double d[3], const double posb[3],
                     const double db[3], double pb, double tb, double xb[6], FrameBar &fb,
                     double sp, double cp, double st, double ct) {
  for (int r = 0; r < 3; ++r) {
    xb[0] += posb[r] * f.U[r];
    xb[1] += posb[r] * f.V[r];
    fb.U[r] += posb[r] * x[0];
    fb.V[r] += posb[r] * x[1];
    fb.c[r] += posb[r];
  }
  const double v[3] = {cp * st, sp * st, ct};
  const double in = rsqrtD(dot(v, v));
  const double pr = dot(d, db);
  double vb[3];
  for (int i = 0; i < 3; ++i) vb[i] = (db[i] - d[i] * pr) * in;
  xb[2] += vb[0] * (-sp * st) + vb[1] * (cp * st);
  xb[3] += vb[0] * (cp * ct) + vb[1] * (sp * ct) - vb[2] * st;
  xb[4] += pb * (-(x[4] > 0. ? 1. : -1.) / (x[4] * x[4]));
  xb[5] += tb;
}

struct Leg {
  double qop, dtds, d37, idt; // idt = 1 / dtds
};
// from ip = 1 / p (the fit's legConstantsIp: one 1/sqrt(1 + (m/p)^2))
KF_HD void legFwdIp(double ip, double q, double mass, Leg &g) {
  g.qop = q * ip;
  const double x = mass * ip, a = 1. + x * x;
#ifdef __CUDA_ARCH__
  const double y = rsqrt(a);
#else
  const double y = 1. / sqrt(a);
#endif
  g.dtds = a * y;
  g.idt = y;
  g.d37 = mass * mass * q * ip * y;
}
KF_HD void legFwd(double p, double q, double mass, Leg &g) { legFwdIp(1. / p, q, mass, g); }
// adjoint of the leg constants w.r.t. p, given ip = 1 / p
KF_HD void legVjpIp(double ip, double q, double mass, const Leg &g, double qopb, double dtdsb,
                    double d37b, double &pb) {
  const double idt = g.idt;
  const double ddt = -(mass * mass) * (ip * ip * ip) * idt;
  pb += qopb * (-q * (ip * ip));
  pb += dtdsb * ddt;
  pb += d37b * (-g.d37 * ip - g.d37 * idt * ddt);
}
KF_HD void legVjp(double p, double q, double mass, const Leg &g, double qopb, double dtdsb,
                  double d37b, double &pb) {
  legVjpIp(1. / p, q, mass, g, qopb, dtdsb, d37b, pb);
}

// ---------------------------------------------------------------------------
// Alignment of a plane: centre shift (dx, dy, dz) and small rotations
// (wx, wy, wz) about the global axes applied to the frame U, V, T.  At zero
// alignment dc/dshift = I and dW/dw_a = e_a x W, so the gradient is
// (cbar, sum_W W x Wbar).
// ---------------------------------------------------------------------------
KF_HD void alignmentGrad(const Frame &f, const FrameBar &b, double g[6]) {
  double r[3], s[3] = {0., 0., 0.};
  cross(f.U, b.U, r);
  for (int i = 0; i < 3; ++i) s[i] += r[i];
  cross(f.V, b.V, r);
  for (int i = 0; i < 3; ++i) s[i] += r[i];
  cross(f.T, b.T, r);
  for (int i = 0; i < 3; ++i) s[i] += r[i];
  for (int i = 0; i < 3; ++i) {
    g[i] = b.c[i];
    g[3 + i] = s[i];
  }
}
// the frame of a plane rotated by small angles w about the global axes
// (R = Rx(wx) Ry(wy) Rz(wz), exact rotation) and shifted: used by tests
KF_HD void alignFrame(const Frame &f, const double a[6], Frame &o) {
  const double cx = cos(a[3]), sx = sin(a[3]), cy = cos(a[4]), sy = sin(a[4]), cz = cos(a[5]),
               sz = sin(a[5]);
  const double R[3][3] = {{cy * cz, -cy * sz, sy},
                          {sx * sy * cz + cx * sz, -sx * sy * sz + cx * cz, -sx * cy},
                          {-cx * sy * cz + sx * sz, cx * sy * sz + sx * cz, cx * cy}};
  for (int i = 0; i < 3; ++i) {
    o.c[i] = f.c[i] + a[i];
    o.U[i] = R[i][0] * f.U[0] + R[i][1] * f.U[1] + R[i][2] * f.U[2];
    o.V[i] = R[i][0] * f.V[0] + R[i][1] * f.V[1] + R[i][2] * f.V[2];
    o.T[i] = R[i][0] * f.T[0] + R[i][1] * f.T[1] + R[i][2] * f.T[2];
  }
}

// ---------------------------------------------------------------------------
// Smoothed chi2 through the closed-form smoother (noise-free RTS: gain =
// J^-1, GainMatrixSmoother.hpp:21-94):
//   xs[n-1] = xf[n-1],  xs[i] = xf[i] + G (xs[i+1] - xp[i+1]),  G = J[i+1]^-1
//   chi2_s = sum over non-outlier states of r^T V^-1 r, r = m - xs[0:2]
// ---------------------------------------------------------------------------
// full 6x6 from the stored 25 entries (rows 0-3,5 x cols 0-4; row 4 = e4,
// column 5 = e5)
KF_HD void jstFull(const double Js[25], double J[6][6]) {
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) J[r][c] = (r == c && (r == 4 || r == 5)) ? 1. : 0.;
  for (int c = 0; c < 5; ++c) {
    J[0][c] = Js[c];
    J[1][c] = Js[5 + c];
    J[2][c] = Js[10 + c];
    J[3][c] = Js[15 + c];
    J[5][c] = Js[20 + c];
  }
  J[4][4] = 1.;
}
// xs <- xf + G (xs_next - xp_next), G given in stored layout
KF_HD void smoothStep(const double Gs[25], const double xf[6], const double xsn[6],
                      const double xpn[6], double xs[6]) {
  double dx[6];
  for (int e = 0; e < 6; ++e) dx[e] = xsn[e] - xpn[e];
  for (int r = 0; r < 6; ++r) {
    if (r == 4) {
      xs[4] = xf[4] + dx[4];
    } else {
      const int gr = (r == 5) ? 4 : r;
      double g = Gs[5 * gr] * dx[0];
      for (int k = 1; k < 5; ++k) g += Gs[5 * gr + k] * dx[k];
      if (r == 5) g += dx[5];
      xs[r] = xf[r] + g;
    }
  }
}
// adjoint of smoothStep: xsb (adjoint of xs) -> xfb, xsnb, xpnb, Gb (stored layout)
KF_HD void smoothStepVjp(const double Gs[25], const double xsn[6], const double xpn[6],
                         const double xsb[6], double xfb[6], double xsnb[6], double xpnb[6],
                         double Gb[25]) {
  double dx[6], dxb[6] = {0., 0., 0., 0., 0., 0.};
  for (int e = 0; e < 6; ++e) dx[e] = xsn[e] - xpn[e];
  for (int r = 0; r < 6; ++r) {
    xfb[r] += xsb[r];
    if (r == 4) {
      dxb[4] += xsb[4];
    } else {
      const int gr = (r == 5) ? 4 : r;
      for (int k = 0; k < 5; ++k) {
        Gb[5 * gr + k] += xsb[r] * dx[k];
        dxb[k] += xsb[r] * Gs[5 * gr + k];
      }
      if (r == 5) dxb[5] += xsb[5];
    }
  }
  for (int e = 0; e < 6; ++e) {
    xsnb[e] += dxb[e];
    xpnb[e] -= dxb[e];
  }
}
// Gb (stored layout, adjoint of G = J^-1) -> Jb (stored layout): Jb = -G^T Gb G^T,
// on the structure G and J share (row 4 = e4, column 5 = e5) and Gb's free
// entries (rows 0-3, 5; columns 0-4): products with the structural zeros and
// ones are not formed (a product with a literal 0 is not free in IEEE FP64)
KF_HD void invVjp(const double Gs[25], const double Gb[25], double Jb[25]) {
  // stored row ri of Gs / Gb / Jb is full row kFree[ri]
  constexpr int kFree[5] = {0, 1, 2, 3, 5};
  // T = G^T B with B = Gb placed on the free entries: T[r][c] = sum over
  // free rows k of G[k][r] B[k][c], c < 5 (B's column 5 is 0); row 5 of T is
  // B's row 5 (G's column 5 is e5)
  double T[6][5];
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) {
      double s = 0.;
      for (int ki = 0; ki < 5; ++ki) s += Gs[5 * ki + r] * Gb[5 * ki + c];
      T[r][c] = s;
    }
  for (int c = 0; c < 5; ++c) T[5][c] = Gb[20 + c];
  // Jb = -T G^T on the free rows, columns 0-4: sum over k < 5 of T[r][k] G[c][k]
  // (T's column 5 is 0); G's row 4 is e4, so column 4 takes T[r][4]
  for (int ri = 0; ri < 5; ++ri) {
    const int r = kFree[ri];
    for (int c = 0; c < 5; ++c) {
      double s;
      if (c == 4) {
        s = T[r][4];
      } else {
        s = 0.;
        for (int k = 0; k < 5; ++k) s += T[r][k] * Gs[5 * c + k];
      }
      Jb[5 * ri + c] -= s;
    }
  }
}

// ---------------------------------------------------------------------------
// Start of the fit: free state and jacToGlobal from the perigee parameters
// (EigenStepper.hpp:40-61, coordinate_transformations.hpp:45-76,
// LineSurface.ipp:63-112,184-198).  Used once per track, so its adjoint is
// taken in forward mode (one dual-number pass per start parameter).
// ---------------------------------------------------------------------------
struct Dual {
  double v, d;
};
KF_HD Dual dl(double v) { return Dual{v, 0.}; }
KF_HD Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
KF_HD Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
KF_HD Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
KF_HD Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
KF_HD Dual operator/(Dual a, Dual b) {
  return Dual{a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)};
}
KF_HD Dual dsqrt(Dual a) {
  const double s = sqrt(a.v);
  return Dual{s, a.d / (2. * s)};
}
KF_HD Dual dsin(Dual a) { return Dual{sin(a.v), cos(a.v) * a.d}; }
KF_HD Dual dcos(Dual a) { return Dual{cos(a.v), -sin(a.v) * a.d}; }
KF_HD Dual dabs(Dual a) { return a.v < 0. ? -a : a; }
KF_HD double val(Dual a) { return a.v; }
KF_HD double val(double a) { return a; }
KF_HD double dsqrt(double a) { return sqrt(a); }
KF_HD double dsin(double a) { return sin(a); }
KF_HD double dcos(double a) { return cos(a); }
KF_HD double dabs(double a) { return fabs(a); }
KF_HD double dl2(double v) { return v; }

template <typename T> struct StartState {
  T pos[3], dir[3], p, t;
  T g03[3][4], g46[3][2];
};

template <typename T>
KF_HD void startFwd(const T sp[6], const double per[3], StartState<T> &o) {
  const T one = T{1.};
  const T pabs = dabs(one / sp[4]);
  const T sph = dsin(sp[2]), cph = dcos(sp[2]), sth = dsin(sp[3]), cth = dcos(sp[3]);
  const T mom[3] = {pabs * sth * cph, pabs * sth * sph, pabs * cth};
  const T rad0 = -mom[1], rad1 = mom[0];
  const T rn = dsqrt(rad0 * rad0 + rad1 * rad1);
  o.pos[0] = T{per[0]} + sp[0] * (rad0 / rn);
  o.pos[1] = T{per[1]} + sp[0] * (rad1 / rn);
  o.pos[2] = (sp[1] + T{per[2]});
  const T pn = dsqrt(mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2]);
  for (int i = 0; i < 3; ++i) o.dir[i] = mom[i] / pn;
  o.p = pn;
  o.t = sp[5];
  const T x = o.dir[0], y = o.dir[1], z = o.dir[2];
  const T cosT = z, sinT = dsqrt(x * x + y * y);
  const T inv = one / sinT;
  const T cosP = x * inv, sinP = y * inv;
  // lineFrame: Y = z axis, X = unit(Y x d), D = X x Y
  const T c0 = -y, c1 = x;
  const T cn = dsqrt(c0 * c0 + c1 * c1);
  const T X[3] = {c0 / cn, c1 / cn, T{0.}};
  const T D[3] = {X[1], -X[0], T{0.}};
  o.g46[0][0] = (-sinT) * sinP;
  o.g46[0][1] = cosT * cosP;
  o.g46[1][0] = sinT * cosP;
  o.g46[1][1] = cosT * sinP;
  o.g46[2][0] = T{0.};
  o.g46[2][1] = -sinT;
  const T ipdn = one / (o.dir[0] * D[0] + o.dir[1] * D[1] + o.dir[2] * D[2]);
  // Y x v = (-v1, v0, 0)
  T dP[3] = {-o.g46[1][0], o.g46[0][0], T{0.}};
  T dT[3] = {-o.g46[1][1], o.g46[0][1], T{0.}};
  const T xp = X[0] * dP[0] + X[1] * dP[1] + X[2] * dP[2];
  const T xt = X[0] * dT[0] + X[1] * dT[1] + X[2] * dT[2];
  const T Y[3] = {T{0.}, T{0.}, one};
  for (int r = 0; r < 3; ++r) {
    dP[r] = dP[r] - xp * X[r];
    dT[r] = dT[r] - xt * X[r];
    o.g03[r][0] = X[r];
    o.g03[r][1] = Y[r];
    o.g03[r][2] = dP[r] * sp[0] * ipdn;
    o.g03[r][3] = dT[r] * sp[0] * ipdn;
  }
}

// adjoints of the start state (pos, dir, p, t, jacToGlobal) -> start parameters
KF_HD void startVjp(const double sp[6], const double per[3], const double posb[3],
                    const double db[3], double pb, double tb, const Gj &Gb, double spb[6]) {
  for (int k = 0; k < 6; ++k) {
    Dual s[6];
    for (int e = 0; e < 6; ++e) s[e] = Dual{sp[e], e == k ? 1. : 0.};
    StartState<Dual> o;
    startFwd<Dual>(s, per, o);
    double g = pb * o.p.d + tb * o.t.d;
    for (int i = 0; i < 3; ++i) g += posb[i] * o.pos[i].d + db[i] * o.dir[i].d;
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 4; ++c) g += Gb.g03[r][c] * o.g03[r][c].d;
      g += Gb.g46[r][0] * o.g46[r][0].d + Gb.g46[r][1] * o.g46[r][1].d;
    }
    spb[k] += g;
  }
}

} // namespace kfa
