// Central finite-difference checks of every vector-Jacobian product in
// kf_adjoint_math.h.  Prints one line per primitive: name, worst relative
// error over random points and random output adjoints.  Built and run by
// tests/test_adjoint_cpu.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <random>
#include <vector>

#include "kf_adjoint_math.h"

using namespace kfa;
using Vec = std::vector<double>;
using Fn = std::function<Vec(const Vec &)>;

static std::mt19937_64 rng(12345);
static double U01() { return std::uniform_real_distribution<double>(0., 1.)(rng); }
static double N01() { return std::normal_distribution<double>(0., 1.)(rng); }

// worst |analytic - fd| / max(|fd|, scale) over the inputs
static double check(const Fn &F, const Vec &x, const Vec &yb, const Vec &xb, double rel = 1e-6) {
  double worst = 0., scale = 0.;
  std::vector<double> fd(x.size());
  for (size_t i = 0; i < x.size(); ++i) {
    const double h = rel * (fabs(x[i]) > 1e-3 ? fabs(x[i]) : 1e-3);
    Vec a = x, b = x;
    a[i] += h;
    b[i] -= h;
    const Vec ya = F(a), yb2 = F(b);
    double s = 0.;
    for (size_t k = 0; k < yb.size(); ++k) s += yb[k] * (ya[k] - yb2[k]);
    fd[i] = s / (2. * h);
    scale = fmax(scale, fabs(fd[i]));
  }
  // error relative to the largest gradient component (FD noise on tiny
  // components is not an error of the product)
  for (size_t i = 0; i < x.size(); ++i) {
    const double e = fabs(xb[i] - fd[i]) / fmax(scale, 1e-300);
    if (getenv("KFA_VERBOSE") && e > 1e-7)
      fprintf(stderr, "  input %zu: analytic %.10e fd %.10e\n", i, xb[i], fd[i]);
    worst = fmax(worst, e);
  }
  return worst;
}

static Vec randv(size_t n) {
  Vec v(n);
  for (auto &x : v) x = N01();
  return v;
}
static void unitDir(double d[3]) {
  // mostly along +x like the telescope tracks
  d[0] = 1.;
  d[1] = 0.1 * (2 * U01() - 1);
  d[2] = 0.1 * (2 * U01() - 1);
  const double n = sqrt(dot(d, d));
  for (int i = 0; i < 3; ++i) d[i] /= n;
}
static double B0[3] = {0., 0., 2. * 0.000299792458};

// ---------------------------------------------------------------------------
static double testStages() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    double d[3];
    unitDir(d);
    Vec x = {d[0], d[1], d[2], (U01() < .5 ? -1 : 1) * (0.1 + U01()), 5. + 60. * U01(),
             B0[0] + 1e-5 * N01(), B0[1] + 1e-5 * N01(), B0[2]};
    Fn F = [](const Vec &v) {
      Stages s;
      stagesFwd(&v[0], v[3], v[4], &v[5], s);
      Vec y;
      for (int i = 0; i < 3; ++i) y.push_back(s.k1[i]);
      for (int i = 0; i < 3; ++i) y.push_back(s.k2[i]);
      for (int i = 0; i < 3; ++i) y.push_back(s.k3[i]);
      for (int i = 0; i < 3; ++i) y.push_back(s.k4[i]);
      y.push_back(s.err);
      return y;
    };
    Vec yb = randv(13);
    Stages s;
    stagesFwd(&x[0], x[3], x[4], &x[5], s);
    double kb[4][3];
    for (int k = 0; k < 4; ++k)
      for (int i = 0; i < 3; ++i) kb[k][i] = yb[3 * k + i];
    Vec xb(8, 0.);
    stagesVjp(&x[0], x[3], x[4], &x[5], s, kb[0], kb[1], kb[2], kb[3], yb[12], &xb[0], xb[3], xb[4],
              &xb[5]);
    // the error estimate is a small difference of stage values: a wider step
    worst = fmax(worst, check(F, x, yb, xb, 1e-4));
  }
  return worst;
}

static double testAccept() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    double d[3];
    unitDir(d);
    Vec x = {100 * N01(), 10 * N01(), N01(), d[0], d[1], d[2], 3. * U01(), 5. + 60. * U01(),
             1. + 0.01 * U01()};
    for (int i = 0; i < 12; ++i) x.push_back(1e-4 * N01());
    auto unpack = [](const Vec &v, Stages &s) {
      for (int i = 0; i < 3; ++i) {
        s.k1[i] = v[9 + i];
        s.k2[i] = v[12 + i];
        s.k3[i] = v[15 + i];
        s.k4[i] = v[18 + i];
      }
    };
    Fn F = [&](const Vec &v) {
      Stages s;
      unpack(v, s);
      Moved m;
      acceptFwd(&v[0], &v[3], v[6], v[7], v[8], s, m);
      Vec y(m.pos, m.pos + 3);
      y.insert(y.end(), m.dir, m.dir + 3);
      y.push_back(m.t);
      return y;
    };
    Vec yb = randv(7);
    Stages s;
    unpack(x, s);
    Moved m;
    acceptFwd(&x[0], &x[3], x[6], x[7], x[8], s, m);
    Vec xb(21, 0.);
    acceptVjp(&x[3], x[7], x[8], s, m, &yb[0], &yb[3], yb[6], &xb[0], &xb[3], xb[6], xb[7], xb[8],
              &xb[9], &xb[12], &xb[15], &xb[18]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testTransport() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    double d[3];
    unitDir(d);
    Vec x = {d[0], d[1], d[2], (U01() < .5 ? -1 : 1) * (0.1 + U01()), 5. + 60. * U01(),
             0.01 * N01(), B0[0] + 1e-5 * N01(), B0[1] + 1e-5 * N01(), B0[2]};
    Fn F = [](const Vec &v) {
      Stages s;
      stagesFwd(&v[0], v[3], v[4], &v[6], s);
      DMat D;
      TransportTmp X;
      transportFwd(&v[0], v[3], v[4], v[5], &v[6], s, D, X);
      Vec y;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) y.push_back(D.DA[i][j]);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) y.push_back(D.DB[i][j]);
      for (int i = 0; i < 3; ++i) y.push_back(D.Da[i]);
      for (int i = 0; i < 3; ++i) y.push_back(D.Dc[i]);
      y.push_back(D.D37);
      return y;
    };
    Vec yb = randv(25);
    Stages s;
    stagesFwd(&x[0], x[3], x[4], &x[6], s);
    DMat D, Db;
    TransportTmp X;
    transportFwd(&x[0], x[3], x[4], x[5], &x[6], s, D, X);
    int k = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Db.DA[i][j] = yb[k++];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Db.DB[i][j] = yb[k++];
    for (int i = 0; i < 3; ++i) Db.Da[i] = yb[k++];
    for (int i = 0; i < 3; ++i) Db.Dc[i] = yb[k++];
    Db.D37 = yb[k++];
    Vec xb(9, 0.);
    double kb[4][3] = {};
    transportVjp(&x[0], x[3], x[4], x[5], &x[6], s, X, Db, &xb[0], xb[3], xb[4], xb[5], &xb[6],
                 kb[0], kb[1], kb[2]);
    stagesVjp(&x[0], x[3], x[4], &x[6], s, kb[0], kb[1], kb[2], kb[3], 0., &xb[0], xb[3], xb[4],
              &xb[6]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static void packJT(const JT &J, Vec &v) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v.push_back(J.A[i][j]);
  for (int i = 0; i < 3; ++i) v.push_back(J.a[i]);
  v.push_back(J.b);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v.push_back(J.B[i][j]);
  for (int i = 0; i < 3; ++i) v.push_back(J.c[i]);
}
static void unpackJT(const double *v, JT &J) {
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J.A[i][j] = v[k++];
  for (int i = 0; i < 3; ++i) J.a[i] = v[k++];
  J.b = v[k++];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J.B[i][j] = v[k++];
  for (int i = 0; i < 3; ++i) J.c[i] = v[k++];
}
static void unpackD(const double *v, DMat &D) {
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) D.DA[i][j] = v[k++];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) D.DB[i][j] = v[k++];
  for (int i = 0; i < 3; ++i) D.Da[i] = v[k++];
  for (int i = 0; i < 3; ++i) D.Dc[i] = v[k++];
  D.D37 = v[k++];
}
static void packD(const DMat &D, Vec &v) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v.push_back(D.DA[i][j]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v.push_back(D.DB[i][j]);
  for (int i = 0; i < 3; ++i) v.push_back(D.Da[i]);
  for (int i = 0; i < 3; ++i) v.push_back(D.Dc[i]);
  v.push_back(D.D37);
}

static double testJtApply() {
  double worst = 0.;
  for (int t = 0; t < 10; ++t) {
    Vec x = randv(50);
    Fn F = [](const Vec &v) {
      DMat D;
      JT J, O;
      unpackD(&v[0], D);
      unpackJT(&v[25], J);
      jtApply(D, J, O);
      Vec y;
      packJT(O, y);
      return y;
    };
    Vec yb = randv(25);
    DMat D, Db;
    JT J, Ob, Jb;
    unpackD(&x[0], D);
    unpackJT(&x[25], J);
    unpackJT(&yb[0], Ob);
    dmZero(Db);
    jtZero(Jb);
    jtApplyVjp(D, J, Ob, Db, Jb);
    Vec xb;
    packD(Db, xb);
    packJT(Jb, xb);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testPath() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    double d[3];
    unitDir(d);
    Vec x = {100 * N01(), 10 * N01(), N01(), d[0], d[1], d[2], 500 + 10 * N01(), N01(), N01(),
             1., 0.01 * N01(), 0.01 * N01()};
    Fn F = [](const Vec &v) { return Vec{pathFwd(&v[0], &v[3], &v[6], &v[9])}; };
    Vec yb = {N01()};
    Vec xb(12, 0.);
    pathVjp(&x[0], &x[3], &x[6], &x[9], yb[0], &xb[0], &xb[3], &xb[6], &xb[9]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testScale() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    Vec x = {1e-4 * (0.02 + 50. * U01())};
    Fn F = [](const Vec &v) {
      double dd;
      return Vec{accScale(v[0], 1e-4, &dd)};
    };
    double dsde;
    accScale(x[0], 1e-4, &dsde);
    Vec yb = {N01()};
    Vec xb = {yb[0] * dsde};
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

// random symmetric positive definite 6x6 (upper triangle)
static void randCov(double C[21]) {
  double A[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) A[i][j] = N01() * (i == j ? 1. : 0.3);
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j) {
      double s = (i == j) ? 0.1 : 0.;
      for (int k = 0; k < 6; ++k) s += A[i][k] * A[j][k];
      C[ut6(i, j)] = s * 1e-3;
    }
}
static void randFrame(Frame &f) {
  // a plane roughly perpendicular to x: T ~ x, U ~ y, V ~ z
  double T[3] = {1., 0.05 * N01(), 0.05 * N01()};
  double n = sqrt(dot(T, T));
  for (int i = 0; i < 3; ++i) T[i] /= n;
  double z[3] = {0., 0., 1.}, U[3], V[3];
  cross(z, T, U);
  n = sqrt(dot(U, U));
  for (int i = 0; i < 3; ++i) U[i] /= n;
  cross(T, U, V);
  for (int i = 0; i < 3; ++i) {
    f.T[i] = T[i];
    f.U[i] = U[i];
    f.V[i] = V[i];
  }
  f.c[0] = 500. + 10 * N01();
  f.c[1] = N01();
  f.c[2] = N01();
}
static void packFrame(const Frame &f, Vec &v) {
  v.insert(v.end(), f.c, f.c + 3);
  v.insert(v.end(), f.U, f.U + 3);
  v.insert(v.end(), f.V, f.V + 3);
  v.insert(v.end(), f.T, f.T + 3);
}
static void unpackFrame(const double *v, Frame &f) {
  for (int i = 0; i < 3; ++i) {
    f.c[i] = v[i];
    f.U[i] = v[3 + i];
    f.V[i] = v[6 + i];
    f.T[i] = v[9 + i];
  }
}
static void packG(const Gj &G, Vec &v) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) v.push_back(G.g03[r][c]);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) v.push_back(G.g46[r][c]);
}
static void unpackG(const double *v, Gj &G) {
  int k = 0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) G.g03[r][c] = v[k++];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) G.g46[r][c] = v[k++];
}

// bound input layout: pos 3, dir 3, p, t, J 25, G 18, dtds, k4 3, C 21, frame 12 (= 90)
static void unpackBound(const Vec &v, BoundIn &in, Frame &f, double q, bool stepped) {
  for (int i = 0; i < 3; ++i) {
    in.pos[i] = v[i];
    in.dir[i] = v[3 + i];
  }
  in.q = q;
  in.p = v[6];
  in.t = v[7];
  unpackJT(&v[8], in.J);
  unpackG(&v[33], in.G);
  in.dtds = v[51];
  for (int i = 0; i < 3; ++i) in.k4[i] = v[52 + i];
  for (int e = 0; e < 21; ++e) in.C[e] = v[55 + e];
  in.stepped = stepped;
  unpackFrame(&v[76], f);
}

static double testBound() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    const bool stepped = (t % 4) != 3;
    const double q = (t % 2) ? 1. : -1.;
    double d[3];
    unitDir(d);
    Frame f;
    randFrame(f);
    Vec x = {f.c[0] + 0.1 * N01(), 10 * N01(), 10 * N01(), d[0], d[1], d[2], 1. + 5. * U01(),
             N01()};
    JT J;
    jtIdentity(J);
    Vec jv;
    packJT(J, jv);
    for (auto &e : jv) e += 0.05 * N01();
    jv[0] += 30.;
    x.insert(x.end(), jv.begin(), jv.end());
    for (int e = 0; e < 18; ++e) x.push_back(N01());
    x.push_back(1. + 0.01 * U01());
    for (int e = 0; e < 3; ++e) x.push_back(1e-4 * N01());
    double C[21];
    randCov(C);
    x.insert(x.end(), C, C + 21);
    packFrame(f, x);
    Fn F = [q, stepped](const Vec &v) {
      BoundIn in;
      Frame fr;
      unpackBound(v, in, fr, q, stepped);
      BoundOut o;
      BoundTmp w;
      boundFwd(in, fr, o, w);
      Vec y(o.pred, o.pred + 6);
      y.insert(y.end(), o.Cp, o.Cp + 21);
      y.insert(y.end(), o.Jst, o.Jst + 25);
      packG(o.G, y);
      return y;
    };
    Vec yb = randv(70);
    BoundIn in;
    Frame fr;
    unpackBound(x, in, fr, q, stepped);
    BoundOut o, ob;
    BoundTmp w;
    boundFwd(in, fr, o, w);
    for (int e = 0; e < 6; ++e) ob.pred[e] = yb[e];
    for (int e = 0; e < 21; ++e) ob.Cp[e] = yb[6 + e];
    for (int e = 0; e < 25; ++e) ob.Jst[e] = yb[27 + e];
    unpackG(&yb[52], ob.G);
    BoundInBar ib;
    FrameBar fb;
    boundInBarZero(ib);
    frameBarZero(fb);
    boundVjp(in, fr, o, w, ob, ib, fb);
    Vec xb(ib.pos, ib.pos + 3);
    xb.insert(xb.end(), ib.dir, ib.dir + 3);
    xb.push_back(ib.p);
    xb.push_back(ib.t);
    packJT(ib.J, xb);
    packG(ib.G, xb);
    xb.push_back(ib.dtds);
    xb.insert(xb.end(), ib.k4, ib.k4 + 3);
    xb.insert(xb.end(), ib.C, ib.C + 21);
    xb.insert(xb.end(), fb.c, fb.c + 3);
    xb.insert(xb.end(), fb.U, fb.U + 3);
    xb.insert(xb.end(), fb.V, fb.V + 3);
    xb.insert(xb.end(), fb.T, fb.T + 3);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testFilter() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    Vec x = randv(6);
    double C[21];
    randCov(C);
    x.insert(x.end(), C, C + 21);
    const double mv[5] = {x[0] + 0.05 * N01(), x[1] + 0.05 * N01(), 2.5e-3, 1e-4, 2.5e-3};
    Fn F = [&mv](const Vec &v) {
      double filt[6], cf[21], chi2;
      FilterTmp w;
      filterFwd(&v[0], &v[6], mv, filt, cf, &chi2, w);
      Vec y(filt, filt + 6);
      y.insert(y.end(), cf, cf + 21);
      return y;
    };
    Vec yb = randv(27);
    double filt[6], cf[21], chi2;
    FilterTmp w;
    filterFwd(&x[0], &x[6], mv, filt, cf, &chi2, w);
    Vec xb(27, 0.);
    filterVjp(&x[6], w, &yb[0], &yb[6], &xb[0], &xb[6]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testUpdate() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    Frame f;
    randFrame(f);
    Vec x = {10 * N01(), 10 * N01(), 0.1 * N01(), 1.5 + 0.1 * N01(),
             (t % 2 ? 1 : -1) * (0.1 + U01()), N01()};
    packFrame(f, x);
    Fn F = [](const Vec &v) {
      Frame fr;
      unpackFrame(&v[6], fr);
      double pos[3], d[3], p, tt;
      updateFwd(fr, &v[0], pos, d, &p, &tt);
      Vec y(pos, pos + 3);
      y.insert(y.end(), d, d + 3);
      y.push_back(p);
      y.push_back(tt);
      return y;
    };
    Vec yb = randv(8);
    Frame fr;
    unpackFrame(&x[6], fr);
    double pos[3], d[3], p, tt, trig[4];
    updateFwd(fr, &x[0], pos, d, &p, &tt, trig);
    Vec xb(6, 0.);
    FrameBar fb;
    frameBarZero(fb);
    updateVjp(fr, &x[0], d, &yb[0], &yb[3], yb[6], yb[7], &xb[0], fb, trig[0], trig[1], trig[2],
              trig[3]);
    xb.insert(xb.end(), fb.c, fb.c + 3);
    xb.insert(xb.end(), fb.U, fb.U + 3);
    xb.insert(xb.end(), fb.V, fb.V + 3);
    xb.insert(xb.end(), fb.T, fb.T + 3);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testLeg() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    const double q = (t % 2) ? 1. : -1., m = 0.1056583755;
    Vec x = {0.5 + 10. * U01()};
    Fn F = [q, m](const Vec &v) {
      Leg g;
      legFwd(v[0], q, m, g);
      return Vec{g.qop, g.dtds, g.d37};
    };
    Vec yb = randv(3);
    Leg g;
    legFwd(x[0], q, m, g);
    Vec xb = {0.};
    legVjp(x[0], q, m, g, yb[0], yb[1], yb[2], xb[0]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

// generic inverse of the structured Jacobian for the test (Gauss-Jordan)
static void invStored(const double Js[25], double Gs[25]) {
  double A[6][12];
  double J[6][6];
  jstFull(Js, J);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 12; ++j) A[i][j] = j < 6 ? J[i][j] : (j - 6 == i ? 1. : 0.);
  for (int c = 0; c < 6; ++c) {
    int p = c;
    for (int r = c + 1; r < 6; ++r)
      if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
    for (int j = 0; j < 12; ++j) std::swap(A[c][j], A[p][j]);
    const double iv = 1. / A[c][c];
    for (int j = 0; j < 12; ++j) A[c][j] *= iv;
    for (int r = 0; r < 6; ++r)
      if (r != c) {
        const double fct = A[r][c];
        for (int j = 0; j < 12; ++j) A[r][j] -= fct * A[c][j];
      }
  }
  const int rows[5] = {0, 1, 2, 3, 5};
  for (int ri = 0; ri < 5; ++ri)
    for (int c = 0; c < 5; ++c) Gs[5 * ri + c] = A[rows[ri]][6 + c];
}

static double testSmooth() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    // x = J stored 25, xf 6, xsn 6, xpn 6
    Vec x;
    for (int e = 0; e < 25; ++e) x.push_back(0.3 * N01());
    x[0] += 1.;
    x[6] += 1.;
    x[12] += 1.;
    x[18] += 1.;
    for (int e = 0; e < 18; ++e) x.push_back(N01());
    Fn F = [](const Vec &v) {
      double G[25], xs[6];
      invStored(&v[0], G);
      smoothStep(G, &v[25], &v[31], &v[37], xs);
      return Vec(xs, xs + 6);
    };
    Vec yb = randv(6);
    double G[25];
    invStored(&x[0], G);
    Vec xb(43, 0.);
    double Gb[25] = {};
    smoothStepVjp(G, &x[31], &x[37], &yb[0], &xb[25], &xb[31], &xb[37], Gb);
    invVjp(G, Gb, &xb[0]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testStart() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    const double per[3] = {0., 0.02 * N01(), 0.02 * N01()};
    Vec x = {0.05 * N01(), 0.05 * N01(), 0.1 * N01(), 1.5708 + 0.1 * N01(),
             (t % 2 ? 1 : -1) * (0.1 + U01()), N01()};
    Fn F = [&per](const Vec &v) {
      StartState<double> o;
      startFwd<double>(&v[0], per, o);
      Vec y(o.pos, o.pos + 3);
      y.insert(y.end(), o.dir, o.dir + 3);
      y.push_back(o.p);
      y.push_back(o.t);
      Gj G;
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 4; ++c) G.g03[r][c] = o.g03[r][c];
        G.g46[r][0] = o.g46[r][0];
        G.g46[r][1] = o.g46[r][1];
      }
      packG(G, y);
      return y;
    };
    Vec yb = randv(26);
    Gj Gb;
    unpackG(&yb[8], Gb);
    Vec xb(6, 0.);
    startVjp(&x[0], per, &yb[0], &yb[3], yb[6], yb[7], Gb, &xb[0]);
    worst = fmax(worst, check(F, x, yb, xb));
  }
  return worst;
}

static double testAlign() {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    Frame f;
    randFrame(f);
    Vec w = randv(12);
    Fn F = [&f, &w](const Vec &a) {
      Frame o;
      alignFrame(f, &a[0], o);
      Vec y;
      packFrame(o, y);
      double s = 0.;
      for (int i = 0; i < 12; ++i) s += w[i] * y[i];
      return Vec{s};
    };
    FrameBar b;
    for (int i = 0; i < 3; ++i) {
      b.c[i] = w[i];
      b.U[i] = w[3 + i];
      b.V[i] = w[6 + i];
      b.T[i] = w[9 + i];
    }
    Vec g(6);
    alignmentGrad(f, b, &g[0]);
    Vec x(6, 0.);
    worst = fmax(worst, check(F, x, Vec{1.}, g, 1e-1)); // angles at 0: absolute step 1e-4
  }
  return worst;
}

// the polynomial uniform-field step equals the stage-by-stage step
static double testPolyEquivalence() {
  double worst = 0.;
  for (int t = 0; t < 50; ++t) {
    double d[3], pos[3] = {100 * N01(), 10 * N01(), N01()}, B[3] = {1e-5 * N01(), 1e-5 * N01(), B0[2]};
    unitDir(d);
    const double q = (t % 2 ? 1 : -1) * (0.1 + U01()), h = 5. + 80. * U01(), dtds = 1.001, d37 = 0.01;
    Stages s;
    stagesFwd(d, q, h, B, s);
    Moved m;
    acceptFwd(pos, d, 0.5, h, dtds, s, m);
    DMat D;
    TransportTmp X;
    transportFwd(d, q, h, d37, B, s, D, X);
    PolyStep w;
    polyTrialFwd(d, q, h, B, w);
    PolyOut o;
    polyAcceptFwd(pos, d, 0.5, q, h, dtds, d37, B, w, o);
    auto rel = [](double a, double b, double sc) { return fabs(a - b) / sc; };
    // the stage-by-stage error estimate carries cancellation noise ~1e-16/x
    worst = fmax(worst, rel(w.err, s.err, s.err) * 1e-4);
    for (int i = 0; i < 3; ++i) {
      worst = fmax(worst, rel(o.pos[i], m.pos[i], 1000.));
      worst = fmax(worst, rel(o.dir[i], m.dir[i], 1.));
      worst = fmax(worst, rel(o.k4[i], s.k4[i], fabs(q) * B0[2]));
      worst = fmax(worst, rel(o.D.Da[i], D.Da[i], h * h * B0[2]));
      worst = fmax(worst, rel(o.D.Dc[i], D.Dc[i], h * B0[2]));
      for (int j = 0; j < 3; ++j) {
        worst = fmax(worst, rel(o.D.DA[i][j], D.DA[i][j], h));
        worst = fmax(worst, rel(o.D.DB[i][j], D.DB[i][j], 1.));
      }
    }
  }
  return worst;
}

// fast: the reverse sweep's 1/|w| by rsqrt (polyAcceptFwd's fastNorm)
static double testPoly(bool fast = false) {
  double worst = 0.;
  for (int t = 0; t < 20; ++t) {
    double d[3];
    unitDir(d);
    // x: pos 3, d 3, t, q, h, dtds, d37, B 3  (= 14)
    Vec x = {100 * N01(), 10 * N01(), N01(), d[0], d[1], d[2], 3. * U01(),
             (t % 2 ? 1 : -1) * (0.1 + U01()), 5. + 60. * U01(), 1. + 0.01 * U01(), 0.01 * N01(),
             1e-5 * N01(), 1e-5 * N01(), B0[2]};
    Fn F = [fast](const Vec &v) {
      PolyStep w;
      polyTrialFwd(&v[3], v[7], v[8], &v[11], w);
      PolyOut o;
      polyAcceptFwd(&v[0], &v[3], v[6], v[7], v[8], v[9], v[10], &v[11], w, o, fast);
      Vec y(o.pos, o.pos + 3);
      y.insert(y.end(), o.dir, o.dir + 3);
      y.push_back(o.t);
      y.push_back(w.err);
      y.insert(y.end(), o.k4, o.k4 + 3);
      packD(o.D, y);
      return y;
    };
    Vec yb = randv(36);
    PolyStep w;
    polyTrialFwd(&x[3], x[7], x[8], &x[11], w);
    PolyOut o;
    polyAcceptFwd(&x[0], &x[3], x[6], x[7], x[8], x[9], x[10], &x[11], w, o, fast);
    DMat Db;
    unpackD(&yb[11], Db);
    Vec xb(14, 0.);
    polyAcceptVjp(&x[3], x[7], x[8], x[9], x[10], &x[11], w, o, &yb[0], &yb[3], yb[6], &yb[8], Db,
                  &xb[0], &xb[3], xb[6], xb[7], xb[8], xb[9], xb[10], &xb[11]);
    polyErrVjp(&x[3], x[7], x[8], &x[11], w, yb[7], &xb[3], xb[7], xb[8], &xb[11]);
    worst = fmax(worst, check(F, x, yb, xb, 1e-5));
  }
  return worst;
}

// trigByAddition against sin and cos of the summed angles; a correction
// above 0.02 rad is refused
static double testTrigAddition() {
  double worst = 0.;
  for (int t = 0; t < 200; ++t) {
    const double phi = 3. * (2. * U01() - 1.), th = 0.1 + 2.9 * U01();
    const double d[3] = {cos(phi) * sin(th), sin(phi) * sin(th), cos(th)};
    const double dphi = 0.02 * (2. * U01() - 1.), dth = 0.02 * (2. * U01() - 1.);
    double tr[4];
    if (!trigByAddition(d, dphi, dth, tr)) return 1.;
    const double ref[4] = {sin(phi + dphi), cos(phi + dphi), sin(th + dth), cos(th + dth)};
    for (int e = 0; e < 4; ++e) worst = fmax(worst, fabs(tr[e] - ref[e]));
  }
  double tr[4];
  const double d[3] = {1., 0., 0.};
  if (trigByAddition(d, 0.03, 0., tr) || trigByAddition(d, 0., -0.03, tr)) return 1.;
  return worst;
}

int main() {
  printf("stages %.3e\n", testStages());
  printf("accept %.3e\n", testAccept());
  printf("transport %.3e\n", testTransport());
  printf("jtapply %.3e\n", testJtApply());
  printf("path %.3e\n", testPath());
  printf("scale %.3e\n", testScale());
  printf("bound %.3e\n", testBound());
  printf("filter %.3e\n", testFilter());
  printf("update %.3e\n", testUpdate());
  printf("leg %.3e\n", testLeg());
  printf("smooth %.3e\n", testSmooth());
  printf("start %.3e\n", testStart());
  printf("align %.3e\n", testAlign());
  printf("polyequiv %.3e\n", testPolyEquivalence());
  printf("poly %.3e\n", testPoly());
  printf("polyfast %.3e\n", testPoly(true));
  printf("trigadd %.3e\n", testTrigAddition());
  return 0;
}
