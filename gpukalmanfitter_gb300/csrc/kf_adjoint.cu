// kf_adjoint.cu — d(total smoothed chi2) / d(plane alignment, start
// parameters, field scale) by a hand-written reverse sweep (FP64, uniform
// field, plane surfaces).
//
// Objective: chi2 = sum over tracks and non-outlier measurement states of
// (m - H x_s)^T V^-1 (m - H x_s), x_s the smoothed parameters of the fit
// (closed-form RTS smoother).  One thread per track, tracks in work-queue
// order (sorted by sequence length and curvature, kfh::sortQueue, so that a
// warp's lanes take similar numbers of RK steps between surfaces); the
// adjoint's own workspace is indexed by queue position (coalesced), inputs,
// outputs and per-track gradient parts by track:
//   A. forward fit (the fit kernel's own lane program, smoothing off) while a
//      hook records the track's tape (step pre-states and trial step sizes,
//      step-size constraint updates, surface events), with a checkpoint of
//      the whole lane before every 5th measurement state;
//   B. smoother and chi2 from the stored states, then the smoother's reverse
//      sweep: adjoints of every state's predicted and filtered parameters and
//      of its bound-to-bound Jacobian;
//   C. the tape swept backwards with the vector-Jacobian products of
//      kf_adjoint_math.h.  A track whose tape ran over its capacity (and
//      every track with kf_config_t.adjoint_tape = 1) instead restores its
//      checkpoints 5-state segment by segment, last first, runs each segment
//      again through the same lane program while the hook records it, and
//      sweeps that.
// The step size is part of the differentiated function: an accepted step's
// size carries its adjoint to the constraint that set it (the distance to the
// next plane, or the accuracy step of an earlier rejected trial, which in
// turn depends on that trial's error estimate).

#include <cuda_runtime.h>

#include <cstring>

#include "kf_adjoint_math.h"
#include "kf_host.h"
#include "kf_kernels.cuh"

using namespace kfh;

namespace kfd {
namespace adj {

constexpr int kEvery = 5;          // measurement states per checkpointed segment
constexpr int kTapeSegment = 3072; // least tape capacity per track: one recomputed segment (doubles)
constexpr int kTapePerState = 256; // tape capacity per track and surface for the forward's tape
// tape capacity per track: the forward's tape of a whole track of S surfaces
// (the workload of 20 planes uses at most ~210 words a state), and never less
// than one segment for a lane that recomputes
__host__ __device__ constexpr int tapeWords(int S) {
  return S * kTapePerState > kTapeSegment ? S * kTapePerState : kTapeSegment;
}
constexpr int kSnapWords = 128;    // doubles per lane checkpoint (visitLane writes 115)
enum { REC_STEP = 1, REC_ACT = 2, REC_HIT = 3 };
constexpr int kStepFixed = 33;     // pos 3, dir 3, t, p, transport Jacobian 25

struct AdjParams {
  const int32_t *perm; // [n] queue position -> track
  double *stateBar;  // [S][37][n] adjoints of predicted, filtered, Jacobian (by position)
  double *xs;        // [S][6][n] smoothed parameters (by position)
  int32_t *info;     // [S][n] plane index | outlier << 8 (by position)
  double *snap;      // [nCk][kSnapWords][n] (by position)
  double *tape;      // [tapeCap][n] (by position: a warp's lanes at the same tape
                     // offset touch one contiguous line)
  int tapeCap;       // tape words per track
  int fwdTape;       // the forward records the whole track's tape
  double *alignPart; // [S][6][n] (by track)
  double *trackFs;   // [n] per-track d chi2 / d field scale (by track)
  double *chi2;      // [n]
  int32_t *status;   // [n]
  double *gradStart; // [6][stride] or null
  double B0[3];      // field value before scaling
  int grad;
};

__device__ __forceinline__ double hdr(int type, int len) { return (double)(type * 65536 + len); }

// a lane's tape: word k at p[k * n]
struct TapeRef {
  const double *p;
  int64_t n;
  // each word is read once: a streaming load, so that the tape passing
  // through does not evict the spilled registers and state arrays from L2
  __device__ __forceinline__ double operator[](int k) const { return __ldcs(p + (int64_t)k * n); }
  __device__ __forceinline__ TapeRef operator+(int k) const { return {p + (int64_t)k * n, n}; }
};

struct TapeHook {
  static constexpr bool kMaterial = false;
  double *tape; // this lane's word 0; word k at tape[k * n]
  int32_t *info;
  int64_t n;
  int top, head, state, plane, cap;
  bool rec, full, over; // recording; a step failed; the tape ran over its capacity

  __device__ __forceinline__ void put(double v) {
    if (top < cap) __stcs(tape + (int64_t)top * n, v); // written once, read once
    else over = true;
    ++top;
  }
  template <class LT> __device__ __forceinline__ void putJ(const LT &L) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) put(L.JA[i][j]);
    for (int i = 0; i < 3; ++i) put(L.Ja[i]);
    put(L.Jb);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) put(L.JB[i][j]);
    for (int i = 0; i < 3; ++i) put(L.Jc[i]);
  }
  template <class LT> __device__ __forceinline__ void stepBegin(const LT &L) {
    if (!rec) return;
    head = top;
    for (int i = 0; i < 3; ++i) put(L.pos[i]);
    for (int i = 0; i < 3; ++i) put(L.dir[i]);
    put(L.t);
    put(L.p);
    putJ(L);
  }
  // the constraint that sets h: the first minimum of the step constraints
  // (ssMin order, forward direction)
  template <class LT> __device__ __forceinline__ void trial(const LT &L, double h) {
    if (!rec) return;
    int idx = 0;
    long long km = okey(L.ss[0]);
    for (int i = 1; i < 4; ++i) {
      const long long k = okey(L.ss[i]);
      if (k < km) {
        km = k;
        idx = i;
      }
    }
    put(h);
    put((double)idx);
  }
  template <class LT> __device__ __forceinline__ void stepEnd(const LT &, bool ok) {
    if (!rec) return;
    if (!ok) full = true; // a failed step has no derivative: the track is dropped
    put(hdr(REC_STEP, top + 1 - head));
  }
  // A navigation constraint is always set from the state the next RK step
  // starts from (a hit happens only on a surface, where the constraint is
  // released instead), so the record keeps the plane only; the reverse sweep
  // takes the state from that step's record.
  template <class LT> __device__ __forceinline__ void actorSet(const LT &, int k) {
    if (!rec) return;
    put((double)k);
    put(hdr(REC_ACT, 2));
  }
  template <class LT> __device__ __forceinline__ void hitBegin(const LT &L, int k) {
    state = L.measStates;
    plane = k;
    if (!rec) return;
    head = top;
    for (int i = 0; i < 3; ++i) put(L.pos[i]);
    for (int i = 0; i < 3; ++i) put(L.dir[i]);
    put(L.p);
    put(L.t);
    putJ(L);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) put(L.g03(r, c));
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 2; ++c) put(L.g46(r, c));
    put(L.stepped ? 1. : 0.);
    put(L.dtds);
    for (int i = 0; i < 3; ++i) put(L.k4[i]);
    for (int e = 0; e < 21; ++e) put(L.cov(e));
    put((double)k);
    put((double)L.measStates);
  }
  __device__ __forceinline__ void hitEnd(bool outlier) {
    info[(int64_t)state * n] = plane | (outlier ? 256 : 0);
    if (!rec) return;
    put(outlier ? 1. : 0.);
    put(hdr(REC_HIT, top + 1 - head));
  }
};

using ALane = Lane<double, TapeHook>;

// ---- checkpoints: every field of the lane and its cold state --------------
// checkpoints are read back only by a track whose tape ran over: streaming
// stores, as for the tape
struct Saver {
  double *p;
  int64_t n;
  int w;
  __device__ void put(double v) { __stcs(p + (int64_t)(w++) * n, v); }
  __device__ void operator()(double &x) { put(x); }
  __device__ void operator()(int &x) { put((double)x); }
  __device__ void operator()(bool &x) { put(x ? 1. : 0.); }
  __device__ void operator()(uint64_t &x) { put(__longlong_as_double((long long)x)); }
  __device__ void operator()(int64_t &x) { put(__longlong_as_double(x)); }
};
struct Loader {
  const double *p;
  int64_t n;
  int w;
  __device__ void operator()(double &x) { x = p[(int64_t)(w++) * n]; }
  __device__ void operator()(int &x) { x = (int)p[(int64_t)(w++) * n]; }
  __device__ void operator()(bool &x) { x = p[(int64_t)(w++) * n] != 0.; }
  __device__ void operator()(uint64_t &x) { x = (uint64_t)__double_as_longlong(p[(int64_t)(w++) * n]); }
  __device__ void operator()(int64_t &x) { x = __double_as_longlong(p[(int64_t)(w++) * n]); }
};
template <class V> __device__ void visitLane(ALane &L, V &v) {
  for (int i = 0; i < 3; ++i) v(L.pos[i]);
  for (int i = 0; i < 3; ++i) v(L.dir[i]);
  v(L.p);
  v(L.q);
  v(L.t);
  v(L.pathAcc);
  for (int i = 0; i < 4; ++i) v(L.ss[i]);
  v(L.ssDir);
  v(L.navDir);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v(L.JA[i][j]);
  for (int i = 0; i < 3; ++i) v(L.Ja[i]);
  v(L.Jb);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v(L.JB[i][j]);
  for (int i = 0; i < 3; ++i) v(L.Jc[i]);
  for (int i = 0; i < 3; ++i) v(L.k4[i]);
  v(L.stepped);
  v(L.qop);
  v(L.dtds);
  v(L.d37);
  v(L.next);
  v(L.current);
  v(L.nSeq);
  v(L.navCache);
  v(L.navCacheSt);
  {
    int64_t x = L.navCacheLim;
    v(x);
    L.navCacheLim = x;
  }
  v(L.mask);
  v(L.nHits);
  v(L.measStates);
  v(L.firstPlane);
  v(L.targetReached);
  v(L.navBreak);
  v(L.smoothed);
  v(L.finished);
  v(L.result);
  v(L.tn);
  v(L.parked);
  v(L.pc);
  v(L.steps);
  v(L.status);
  v(L.rkSteps);
  v(L.rkTrials);
  v(L.chi2);
  for (int i = 0; i < 3; ++i) v(L.perigee[i]);
  v(L.idx);
  v(L.wsIdx);
  for (int e = 0; e < 21; ++e) {
    double x = L.cov(e);
    v(x);
    L.cov(e) = x;
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) {
      double x = L.g03(r, c);
      v(x);
      L.g03(r, c) = x;
    }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) {
      double x = L.g46(r, c);
      v(x);
      L.g46(r, c) = x;
    }
}

__device__ __forceinline__ bool hitPending(const ALane &L) {
  return L.parked && L.current >= 0 && !L.smoothed && !L.finished &&
         ((L.mask >> L.current) & 1ull);
}

// Run the lane program of every lane of the warp (all 32 lanes call it) until
// each is done or parked before the hit event of measurement state stopAt
// (stopAt < 0: never).  As in the fit kernel, lanes step independently and
// run their surface events together once every lane waits.  With ck (the
// forward of a gradient run), a lane saves itself before the hit events of
// states 5, 10, ...: a lane whose tape ran over its capacity recomputes its
// segments from there.
__device__ void runWarp(ALane &L, const Params &P, const PlaneD *sp, const AdjParams &A,
                        int stopAt, bool ck) {
  bool stopped = false;
  for (;;) {
    if (!L.parked && !stopped && L.pc != PC_DONE) advance(L, P, sp);
    if (L.parked && !stopped && hitPending(L) && L.measStates == stopAt) stopped = true;
    const bool waiting = L.parked || stopped || L.pc == PC_DONE;
    if (__all_sync(0xffffffffu, waiting)) {
      if (L.parked && !stopped) {
        if (ck && hitPending(L) && L.measStates > 0 && L.measStates % kEvery == 0) {
          Saver s{A.snap + (int64_t)(L.measStates / kEvery - 1) * kSnapWords * P.n + L.wsIdx, P.n, 0};
          visitLane(L, s);
        }
        runEvent(L, P, sp);
      }
      if (__all_sync(0xffffffffu, stopped || L.pc == PC_DONE)) return;
    }
  }
}

// ---- the running adjoint of the lane state ---------------------------------
struct Adj {
  double pos[3], dir[3], p, t;
  kfa::JT J;
  kfa::Gj G;
  double C[21];
  double k4[3];
  double ssAcc, ssAct;   // adjoints of the accuracy and navigation step constraints
  double qop, dtds, d37; // adjoints of the per-leg constants
  double B[3];           // adjoint of the field vector
};
__device__ void adjZero(Adj &R) {
  for (int i = 0; i < 3; ++i) R.pos[i] = R.dir[i] = R.k4[i] = R.B[i] = 0.;
  R.p = R.t = R.ssAcc = R.ssAct = R.qop = R.dtds = R.d37 = 0.;
  kfa::jtZero(R.J);
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) R.G.g03[r][c] = 0.;
    R.G.g46[r][0] = R.G.g46[r][1] = 0.;
  }
  for (int e = 0; e < 21; ++e) R.C[e] = 0.;
}

__device__ __forceinline__ void toFrame(const PlaneD &pl, kfa::Frame &f) {
  for (int i = 0; i < 3; ++i) {
    f.c[i] = pl.c[i];
    f.U[i] = pl.U[i];
    f.V[i] = pl.V[i];
    f.T[i] = pl.T[i];
  }
}
__device__ __forceinline__ void addAlign(const AdjParams &A, int64_t n, int64_t i, int k,
                                         const kfa::Frame &f, const kfa::FrameBar &fb) {
  double g[6];
  kfa::alignmentGrad(f, fb, g);
  for (int a = 0; a < 6; ++a) A.alignPart[((int64_t)k * 6 + a) * n + i] += g[a];
}
__device__ __forceinline__ void readJT(TapeRef w, kfa::JT &J) {
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J.A[i][j] = w[k++];
  for (int i = 0; i < 3; ++i) J.a[i] = w[k++];
  J.b = w[k++];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J.B[i][j] = w[k++];
  for (int i = 0; i < 3; ++i) J.c[i] = w[k++];
}
// the adjoint of a step-size value goes to the constraint that set it
__device__ __forceinline__ void routeStep(Adj &R, int idx, double hb) {
  if (idx == kAccuracy) R.ssAcc += hb;
  else if (idx == kActor) R.ssAct += hb; // navDir = +1 on the forward leg
}

// reverse of one RK step record (the uniform-field step of the fit,
// kfa::polyAcceptFwd, and the error estimates of its rejected trials)
// g / gp: the leg constants of momentum gp, kept across the steps of a leg
__device__ void reverseStep(TapeRef w, int len, Adj &R, const Params &P, double q,
                            kfa::Leg &g, double &gp) {
  const double pos[3] = {w[0], w[1], w[2]}, dir[3] = {w[3], w[4], w[5]};
  const double t = w[6], p = w[7];
  kfa::JT J0;
  readJT(w + 8, J0);
  const int T = (len - kStepFixed - 1) / 2;
  const TapeRef tr = w + kStepFixed;
  if (p != gp) {
    kfa::legFwd(p, q, P.mass, g);
    gp = p;
  }
  const double *B = P.field.B;
  const double h = tr[2 * (T - 1)];
  kfa::PolyStep ps;
  kfa::polyPrep(dir, B, ps);
  kfa::polyCoef(g.qop, h, ps);
  kfa::PolyOut o;
  kfa::polyAcceptFwd(pos, dir, t, g.qop, h, g.dtds, g.d37, B, ps, o, true);
  // J' = D J
  kfa::DMat Db;
  kfa::dmZero(Db);
  kfa::JT Jb0;
  kfa::jtZero(Jb0);
  kfa::jtApplyVjp(o.D, J0, R.J, Db, Jb0);
  double posb[3] = {0., 0., 0.}, dirb[3] = {0., 0., 0.}, tb = 0., hb = 0.;
  kfa::polyAcceptVjp(dir, g.qop, h, g.dtds, g.d37, B, ps, o, R.pos, R.dir, R.t, R.k4, Db, posb,
                     dirb, tb, R.qop, hb, R.dtds, R.d37, R.B);
  routeStep(R, (int)tr[2 * (T - 1) + 1], hb);
  // rejected trials, last first: each set the accuracy constraint from its
  // error estimate
  for (int k = T - 2; k >= 0; --k) {
    const double gacc = R.ssAcc;
    R.ssAcc = 0.;
    if (gacc == 0.) continue;
    const double ht = tr[2 * k];
    kfa::polyCoef(g.qop, ht, ps);
    double dsde;
    const double sc = kfa::accScale(ps.err, P.tol, &dsde);
    double htb = gacc * sc;
    kfa::polyErrVjp(dir, g.qop, ht, B, ps, gacc * ht * dsde, dirb, R.qop, htb, R.B);
    routeStep(R, (int)tr[2 * k + 1], htb);
  }
  for (int i = 0; i < 3; ++i) {
    R.pos[i] = posb[i];
    R.dir[i] = dirb[i];
    R.k4[i] = 0.;
  }
  R.t = tb;
  R.J = Jb0;
}

// reverse of a navigation step-constraint update (distance to plane k from
// the state pos, dir that the following RK step starts from)
__device__ void reverseAct(TapeRef w, const double pos[3], const double dir[3], Adj &R,
                           const PlaneD *sp, const AdjParams &A, int64_t n, int64_t i) {
  if (R.ssAct == 0.) return;
  const int k = (int)w[0];
  kfa::Frame f;
  toFrame(sp[k], f);
  kfa::FrameBar fb;
  kfa::frameBarZero(fb);
  kfa::pathVjp(pos, dir, f.c, f.T, R.ssAct, R.pos, R.dir, fb.c, fb.T);
  R.ssAct = 0.;
  addAlign(A, n, i, k, f, fb);
}

// reverse of a surface event with a hit: bound state (prediction, covariance
// transport, jacToGlobal), gain update, stepper update
__device__ void reverseHit(TapeRef w, Adj &R, const Params &P, const PlaneD *sp,
                           const AdjParams &A, int64_t u, int64_t i, double q) {
  const int64_t n = P.n;
  kfa::BoundIn in;
  for (int e = 0; e < 3; ++e) {
    in.pos[e] = w[e];
    in.dir[e] = w[3 + e];
  }
  in.q = q;
  in.p = w[6];
  in.t = w[7];
  readJT(w + 8, in.J);
  {
    int k = 33;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) in.G.g03[r][c] = w[k++];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 2; ++c) in.G.g46[r][c] = w[k++];
  }
  in.stepped = w[51] != 0.;
  in.dtds = w[52];
  for (int e = 0; e < 3; ++e) in.k4[e] = w[53 + e];
  for (int e = 0; e < 21; ++e) in.C[e] = w[56 + e];
  const int k = (int)w[77], s = (int)w[78];
  const bool outlier = w[79] != 0.;
  kfa::Frame f;
  toFrame(sp[k], f);
  kfa::BoundOut o, ob;
  kfa::BoundTmp bt;
  kfa::boundFwd(in, f, o, bt, false);
  // predicted parameters as the forward stored them, and below the smoother
  // adjoints of this state: read once here, long after they were written
  // (streaming loads)
  auto WS = [&](int e) { return __ldcs(P.ws + ((int64_t)s * kStateStride + e) * n + u); };
  for (int e = 0; e < 6; ++e) o.pred[e] = WS(e);
  const double *sb = A.stateBar + u;
  auto SB = [&](int e) { return __ldcs(sb + ((int64_t)s * kStateStride + e) * n); };
  for (int e = 0; e < 6; ++e) ob.pred[e] = SB(e);
  for (int e = 0; e < 25; ++e) ob.Jst[e] = SB(12 + e);
  ob.G = R.G;
  for (int e = 0; e < 21; ++e) ob.Cp[e] = 0.;
  kfa::FrameBar fb;
  kfa::frameBarZero(fb);
  if (!outlier) {
    const double *mp = P.meas + (size_t)k * 5 * P.stride + i;
    const double mv[5] = {mp[0], mp[P.stride], mp[2 * P.stride], mp[3 * P.stride],
                          mp[4 * P.stride]};
    double filt[6], cf[21], chi2;
    kfa::FilterTmp fw;
    kfa::filterFwd(o.pred, o.Cp, mv, filt, cf, &chi2, fw);
    // the stepper update as the fit does it: the filtered angles' sines and
    // cosines by angle addition from the predicted direction, the leg
    // constants from 1/p = |q/p|
    double pos1[3], dir1[3], p1, t1, trig[4];
    if (!kfa::trigByAddition(in.dir, filt[2] - o.pred[2], filt[3] - o.pred[3], trig)) {
      kfa::sinCos(filt[2], trig[0], trig[1]);
      kfa::sinCos(filt[3], trig[2], trig[3]);
    }
    kfa::updateFwdTrig(f, filt, trig, pos1, dir1, &p1, &t1);
    kfa::Leg g;
    const double ip1 = fabs(filt[4]);
    kfa::legFwdIp(ip1, q, P.mass, g);
    double pb = R.p;
    kfa::legVjpIp(ip1, q, P.mass, g, R.qop, R.dtds, R.d37, pb);
    R.qop = R.dtds = R.d37 = 0.;
    double filtb[6];
    for (int e = 0; e < 6; ++e) filtb[e] = SB(6 + e);
    kfa::updateVjp(f, filt, dir1, R.pos, R.dir, pb, R.t, filtb, fb, trig[0], trig[1], trig[2],
                   trig[3]);
    kfa::filterVjp(o.Cp, fw, filtb, R.C, ob.pred, ob.Cp);
    for (int e = 0; e < 3; ++e) R.pos[e] = R.dir[e] = 0.;
    R.p = R.t = 0.;
  } else {
    // filtered = predicted; the stepper keeps the predicted state and covariance
    for (int e = 0; e < 6; ++e) ob.pred[e] += SB(6 + e);
    for (int e = 0; e < 21; ++e) ob.Cp[e] = R.C[e];
  }
  kfa::BoundInBar ib;
  kfa::boundInBarZero(ib);
  kfa::boundVjp(in, f, o, bt, ob, ib, fb);
  for (int e = 0; e < 3; ++e) {
    R.pos[e] += ib.pos[e];
    R.dir[e] += ib.dir[e];
    R.k4[e] = ib.k4[e];
  }
  R.p += ib.p;
  R.t += ib.t;
  R.dtds += ib.dtds;
  R.J = ib.J;
  R.G = ib.G;
  for (int e = 0; e < 21; ++e) R.C[e] = ib.C[e];
  addAlign(A, n, i, k, f, fb);
}

// Sweep the tapes of all lanes backwards together: step and navigation
// records whenever a lane has one on top, surface events once every lane with
// work has one on top.  Returns false for a malformed tape.
__device__ bool reverseWarp(TapeRef tape, int top, Adj &R, const Params &P,
                            const PlaneD *sp, const AdjParams &A, int64_t u, int64_t i, double q) {
  bool bad = false;
  double cpos[3] = {0., 0., 0.}, cdir[3] = {0., 0., 0.}; // pre-state of the step after
  kfa::Leg leg;
  double legP = -1.;
  for (;;) {
    int type = 0, len = 0;
    if (top > 0 && !bad) {
      const int h = (int)tape[top - 1];
      type = h >> 16;
      len = h & 0xffff;
      if (len < 2 || len > top || type < REC_STEP || type > REC_HIT) {
        bad = true;
        type = 0;
      }
    }
    if (__any_sync(0xffffffffu, type == REC_STEP || type == REC_ACT)) {
      if (type == REC_STEP) {
        const TapeRef w = tape + (top - len);
        reverseStep(w, len, R, P, q, leg, legP);
        for (int e = 0; e < 3; ++e) {
          cpos[e] = w[e];
          cdir[e] = w[3 + e];
        }
      } else if (type == REC_ACT) {
        reverseAct(tape + (top - len), cpos, cdir, R, sp, A, P.n, i);
      }
      if (type == REC_STEP || type == REC_ACT) top -= len;
    } else {
      if (!__any_sync(0xffffffffu, type == REC_HIT)) break;
      if (type == REC_HIT) {
        reverseHit(tape + (top - len), R, P, sp, A, u, i, q);
        top -= len;
      }
    }
  }
  return !bad;
}

// smoothed chi2 of one track from its stored states; with grad, the adjoints
// of every state's predicted and filtered parameters and Jacobian
__device__ double smoothChi2(const Params &P, const AdjParams &A, int64_t u, int64_t i, int ns,
                             bool grad) {
  const int64_t n = P.n;
  auto WS = [&](int s, int e) { return P.ws[((int64_t)s * kStateStride + e) * n + u]; };
  auto XS = [&](int s, int e) -> double & { return A.xs[((int64_t)s * 6 + e) * n + u]; };
  auto SB = [&](int s, int e) -> double & { return A.stateBar[((int64_t)s * kStateStride + e) * n + u]; };
  double xs[6];
  for (int e = 0; e < 6; ++e) xs[e] = WS(ns - 1, 6 + e);
  for (int e = 0; e < 6; ++e) XS(ns - 1, e) = xs[e];
  for (int s = ns - 2; s >= 0; --s) {
    double Jn[25], G[25], xf[6], xp[6], xn[6];
    for (int e = 0; e < 25; ++e) Jn[e] = WS(s + 1, 12 + e);
    for (int e = 0; e < 6; ++e) {
      xf[e] = WS(s, 6 + e);
      xp[e] = WS(s + 1, e);
      xn[e] = xs[e];
    }
    invJacobian(Jn, G);
    kfa::smoothStep(G, xf, xn, xp, xs);
    for (int e = 0; e < 6; ++e) XS(s, e) = xs[e];
    // the reverse pass below takes the gain from here: the Jacobian-adjoint
    // slots of state s + 1 hold it until that pass writes the adjoint there
    if (grad)
      for (int e = 0; e < 25; ++e) SB(s + 1, 12 + e) = G[e];
  }
  // chi2 terms and their adjoints d chi2 / d xs = -2 V^-1 r (rows 0, 1)
  double chi2 = 0.;
  auto term = [&](int s, double g[2]) {
    g[0] = g[1] = 0.;
    const int inf = A.info[(int64_t)s * n + u];
    if (inf & 256) return;
    const int k = inf & 255;
    const double *mp = P.meas + (size_t)k * 5 * P.stride + i;
    const double v00 = mp[2 * P.stride], v01 = mp[3 * P.stride], v11 = mp[4 * P.stride];
    const double r0 = mp[0] - XS(s, 0), r1 = mp[P.stride] - XS(s, 1);
    const double det = v00 * v11 - v01 * v01;
    const double idet = 1. / det;
    const double w0 = (v11 * r0 - v01 * r1) * idet, w1 = (v00 * r1 - v01 * r0) * idet;
    chi2 += r0 * w0 + r1 * w1;
    g[0] = -2. * w0;
    g[1] = -2. * w1;
  };
  if (!grad) {
    double g[2];
    for (int s = 0; s < ns; ++s) term(s, g);
    return chi2;
  }
  for (int s = 0; s < ns; ++s)
    for (int e = 0; e < (s == 0 ? kStateStride : 12); ++e) SB(s, e) = 0.;
  double xsb[6] = {0., 0., 0., 0., 0., 0.}, g[2];
  term(0, g);
  xsb[0] = g[0];
  xsb[1] = g[1];
  for (int s = 0; s + 1 < ns; ++s) {
    double G[25], Gb[25], Jb[25], xn[6], xp[6], xfb[6], xnb[6], xpb[6];
    for (int e = 0; e < 25; ++e) {
      G[e] = SB(s + 1, 12 + e);
      Gb[e] = Jb[e] = 0.;
    }
    for (int e = 0; e < 6; ++e) {
      xn[e] = XS(s + 1, e);
      xp[e] = WS(s + 1, e);
      xfb[e] = xnb[e] = xpb[e] = 0.;
    }
    kfa::smoothStepVjp(G, xn, xp, xsb, xfb, xnb, xpb, Gb);
    kfa::invVjp(G, Gb, Jb);
    for (int e = 0; e < 6; ++e) {
      SB(s, 6 + e) += xfb[e];
      SB(s + 1, e) += xpb[e];
    }
    for (int e = 0; e < 25; ++e) SB(s + 1, 12 + e) = Jb[e];
    term(s + 1, g);
    for (int e = 0; e < 6; ++e) xsb[e] = xnb[e];
    xsb[0] += g[0];
    xsb[1] += g[1];
  }
  for (int e = 0; e < 6; ++e) SB(ns - 1, 6 + e) += xsb[e];
  return chi2;
}

__device__ void zeroTrack(const Params &P, const AdjParams &A, int64_t i) {
  A.chi2[i] = 0.;
  A.trackFs[i] = 0.;
  for (int64_t k = 0; k < (int64_t)P.nSurf * 6; ++k) A.alignPart[k * P.n + i] = 0.;
  if (A.gradStart)
    for (int e = 0; e < 6; ++e) A.gradStart[(int64_t)e * P.stride + i] = 0.;
}

#ifndef KF_ADJ_MIN_BLOCKS
#define KF_ADJ_MIN_BLOCKS 2
#endif
__global__ void __launch_bounds__(kLaneSlots, KF_ADJ_MIN_BLOCKS)
    adjointKernel(const __grid_constant__ Params P, const __grid_constant__ AdjParams A) {
  __shared__ PlaneD sp[KF_MAX_PLANES];
  for (int k = threadIdx.x; k < P.nSurf; k += blockDim.x) sp[k] = P.planes[k];
  __syncthreads();
  // every lane stays to the end: the lane program and the reverse sweep run
  // warp-synchronously (idle lanes carry no work)
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; // queue position
  const bool valid = u < P.n;
  const int64_t i = valid ? (int64_t)A.perm[u] : 0;                 // track
  ALane L;
  L.hook.tape = A.tape + (valid ? u : 0);
  L.hook.info = A.info + (valid ? u : 0);
  L.hook.n = P.n;
  L.hook.top = L.hook.head = L.hook.state = L.hook.plane = 0;
  L.hook.cap = A.tapeCap;
  L.hook.rec = false;
  L.hook.full = L.hook.over = false;
  if (valid) zeroTrack(P, A, i);
  // ---- A: forward fit with checkpoints and the tape (recording from before
  // initLane, which already sets the step constraint towards the first plane)
  L.hook.rec = valid && A.grad != 0 && A.fwdTape != 0;
  initLane(L, P, sp, valid ? i : -1, valid ? u : 0);
  runWarp(L, P, sp, A, -1, A.grad != 0);
  const int ns = L.measStates;
  const bool ok = valid && L.status == KF_TRACK_OK && ns > 0;
  if (valid) A.status[i] = L.status;
  // ---- B: smoothed chi2 (and the smoother's adjoints)
  if (ok) A.chi2[i] = smoothChi2(P, A, u, i, ns, A.grad != 0);
  if (!A.grad) return;
  // ---- C: the reverse sweep.  A lane whose forward tape holds the whole
  // track sweeps it in one pass (at its last segment's turn); a lane whose
  // tape ran over recomputes its segments from the checkpoints, last first,
  // each onto the start of its tape, and sweeps them one by one.
  Adj R;
  adjZero(R);
  const double q = L.q;
  const int nseg = ok ? (ns - 1) / kEvery + 1 : 0;
  const int maxSeg = __reduce_max_sync(0xffffffffu, nseg);
  const bool fwdTaped = A.fwdTape && !L.hook.over;
  const int fwdTop = L.hook.top;
  bool failed = ok && L.hook.full;
  for (int c = maxSeg - 1; c >= 0; --c) {
    const bool act = ok && !failed && c < nseg;
    const bool recompute = act && !fwdTaped;
    L.hook.rec = recompute;
    if (!recompute) {
      L.pc = PC_DONE;
      L.parked = false;
    } else {
      L.hook.top = 0;
      L.hook.over = false;
      if (c == 0) {
        initLane(L, P, sp, i, u);
      } else {
        Loader ld{A.snap + (int64_t)(c - 1) * kSnapWords * P.n + u, P.n, 0};
        visitLane(L, ld);
      }
    }
    runWarp(L, P, sp, A, (c + 1) * kEvery, false);
    if (recompute && (L.hook.full || L.hook.over)) failed = true;
    const bool sweep = act && !failed && (recompute || c == nseg - 1);
    const int top = recompute ? L.hook.top : fwdTop;
    if (!reverseWarp(TapeRef{L.hook.tape, P.n}, sweep ? top : 0, R, P, sp, A, u, i, q) && sweep)
      failed = true;
  }
  if (!ok) return;
  if (failed) {
    A.status[i] = KF_TRACK_ADJOINT_FAILED;
    zeroTrack(P, A, i);
    return;
  }
  // ---- start parameters: the leg constants belong to the start momentum
  double sp0[6];
  for (int e = 0; e < 6; ++e) sp0[e] = P.start[(int64_t)e * P.stride + i];
  double per[3];
  for (int e = 0; e < 3; ++e) per[e] = P.perigee[(int64_t)e * P.stride + i];
  kfa::StartState<double> st;
  kfa::startFwd<double>(sp0, per, st);
  kfa::Leg g;
  kfa::legFwd(st.p, q, P.mass, g);
  kfa::legVjp(st.p, q, P.mass, g, R.qop, R.dtds, R.d37, R.p);
  double spb[6] = {0., 0., 0., 0., 0., 0.};
  kfa::startVjp(sp0, per, R.pos, R.dir, R.p, R.t, R.G, spb);
  if (A.gradStart)
    for (int e = 0; e < 6; ++e) A.gradStart[(int64_t)e * P.stride + i] = spb[e];
  A.trackFs[i] = R.B[0] * A.B0[0] + R.B[1] * A.B0[1] + R.B[2] * A.B0[2];
}

// deterministic sums over tracks: one CTA per output value
__global__ void __launch_bounds__(256) reduceTracks(const double *src, int64_t n, int nOut,
                                                    double *dst) {
  __shared__ double part[256];
  const int o = blockIdx.x;
  if (o >= nOut) return;
  double s = 0.;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += src[(int64_t)o * n + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) part[threadIdx.x] += part[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) dst[o] = part[0];
}

size_t alignUp(size_t x) { return (x + 255) & ~(size_t)255; }

struct AdjLayout {
  size_t ws, stateBar, xs, info, snap, tape, alignPart, trackFs, perm, hist, offs, total;
};
// tape words per track for kf_config_t.adjoint_tape
int tapeCapacity(int mode, int32_t S) { return mode == 1 ? kTapeSegment : tapeWords(S); }

AdjLayout adjLayout(int64_t n, int32_t S, int mode) {
  AdjLayout L{};
  size_t o = 0;
  auto take = [&](size_t b) {
    const size_t at = o;
    o = alignUp(o + b);
    return at;
  };
  const int nCk = (S - 1) / kEvery; // checkpoints before states 5, 10, ... < S
  L.ws = take(wsBytes(n, S, false));
  L.stateBar = take((size_t)S * kStateStride * n * 8);
  L.xs = take((size_t)S * 6 * n * 8);
  L.info = take((size_t)S * n * 4);
  L.snap = take((size_t)(nCk > 0 ? nCk : 1) * kSnapWords * n * 8);
  L.tape = take((size_t)tapeCapacity(mode, S) * n * 8);
  L.alignPart = take((size_t)S * 6 * n * 8);
  L.trackFs = take((size_t)n * 8);
  L.perm = take((size_t)n * 4);
  L.hist = take((size_t)kSortBuckets * 4);
  L.offs = take((size_t)kSortBuckets * 4);
  L.total = o;
  return L;
}

} // namespace adj
} // namespace kfd

using namespace kfd;
using namespace kfd::adj;

extern "C" {

size_t kf_adjoint_workspace_size(const kf_config_t *cfg, int64_t n_tracks, int32_t n_surfaces) {
  if (n_tracks <= 0 || n_surfaces <= 0) return 0;
  return adjLayout(n_tracks, n_surfaces, cfg ? cfg->adjoint_tape : 0).total;
}

int32_t kf_adjoint_batch(const kf_inputs_t *in, kf_adjoint_outputs_t *out, const kf_config_t *cfg,
                         const kf_geometry_t *geo, const kf_field_t *field,
                         int32_t compute_gradient, void *workspace, size_t workspace_bytes,
                         void *stream) {
  HostRange range("kf_adjoint_batch");
  int32_t rc = checkCommon(in, cfg, geo, field);
  if (rc) return rc;
  if (!out || !out->chi2 || !out->status)
    return fail(KF_ERR_INVALID_ARGUMENT, "missing chi2/status output%s");
  if (cfg->precision != KF_PRECISION_FP64)
    return fail(KF_ERR_UNSUPPORTED, "the adjoint is FP64 only%s");
  if (field->kind != KF_FIELD_CONSTANT)
    return fail(KF_ERR_UNSUPPORTED, "the adjoint supports a uniform field only%s");
  if (!cfg->faithful_jacobian)
    return fail(KF_ERR_UNSUPPORTED, "the adjoint follows faithful_jacobian = 1 only%s");
  if (cfg->material_effects && geo->material)
    return fail(KF_ERR_UNSUPPORTED, "the adjoint has no material effects%s");
  if (cfg->adjoint_tape != 0 && cfg->adjoint_tape != 1)
    return fail(KF_ERR_INVALID_ARGUMENT, "adjoint_tape must be 0 or 1%s");
  const int64_t n = in->n_tracks;
  const int32_t S = in->n_surfaces;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    cudaError_t e = cudaSuccess;
    if (out->grad_align) e = cudaMemsetAsync(out->grad_align, 0, (size_t)S * 6 * 8, s);
    if (e == cudaSuccess && out->grad_field_scale) e = cudaMemsetAsync(out->grad_field_scale, 0, 8, s);
    if (e == cudaSuccess && out->chi2_total) e = cudaMemsetAsync(out->chi2_total, 0, 8, s);
    return e == cudaSuccess ? KF_SUCCESS : cudaFail(e, "zero outputs");
  }
  if (!in->meas || !in->start_params || !in->start_cov || !in->perigee)
    return fail(KF_ERR_INVALID_ARGUMENT, "missing input array%s");
  const AdjLayout L = adjLayout(n, S, cfg->adjoint_tape);
  if (!workspace || workspace_bytes < L.total)
    return fail(KF_ERR_WORKSPACE_TOO_SMALL, "workspace smaller than kf_adjoint_workspace_size()%s");
  char *base = static_cast<char *>(workspace);
  kf_config_t c = *cfg;
  c.smoothing = 0; // the adjoint runs its own smoother on the stored states
  kf_outputs_t none;
  std::memset(&none, 0, sizeof(none));
  Params P;
  fillParams(P, in, &none, &c, geo, field, base + L.ws);
  AdjParams A;
  std::memset(&A, 0, sizeof(A));
  A.perm = reinterpret_cast<const int32_t *>(base + L.perm);
  A.stateBar = reinterpret_cast<double *>(base + L.stateBar);
  A.xs = reinterpret_cast<double *>(base + L.xs);
  A.info = reinterpret_cast<int32_t *>(base + L.info);
  A.snap = reinterpret_cast<double *>(base + L.snap);
  A.tape = reinterpret_cast<double *>(base + L.tape);
  A.tapeCap = tapeCapacity(cfg->adjoint_tape, S);
  A.fwdTape = cfg->adjoint_tape == 0;
  A.alignPart = reinterpret_cast<double *>(base + L.alignPart);
  A.trackFs = (compute_gradient && out->grad_field_scale_track)
                  ? out->grad_field_scale_track
                  : reinterpret_cast<double *>(base + L.trackFs);
  A.chi2 = out->chi2;
  A.status = out->status;
  A.gradStart = compute_gradient ? out->grad_start : nullptr;
  for (int a = 0; a < 3; ++a) A.B0[a] = field->value[a];
  A.grad = compute_gradient != 0;
  rc = sortQueue(P, reinterpret_cast<int32_t *>(base + L.hist),
                 reinterpret_cast<int32_t *>(base + L.offs),
                 reinterpret_cast<int32_t *>(base + L.perm), s);
  if (rc) return rc;
  const unsigned grid = (unsigned)((n + kLaneSlots - 1) / kLaneSlots);
  adjointKernel<<<grid, kLaneSlots, coldStateBytes<double>(), s>>>(P, A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cudaFail(e, "adjoint kernel launch");
  if (compute_gradient && out->grad_align) reduceTracks<<<S * 6, 256, 0, s>>>(A.alignPart, n, S * 6, out->grad_align);
  if (compute_gradient && out->grad_field_scale) reduceTracks<<<1, 256, 0, s>>>(A.trackFs, n, 1, out->grad_field_scale);
  if (out->chi2_total) reduceTracks<<<1, 256, 0, s>>>(A.chi2, n, 1, out->chi2_total);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cudaFail(e, "adjoint reduction launch");
  return KF_SUCCESS;
}

} // extern "C"
