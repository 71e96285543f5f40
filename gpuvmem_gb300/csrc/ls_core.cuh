// linmin's line search (src/linmin.cu:52-110) on the GPU: the bracketing
// step (src/mnbrak.cu:44-98) and Brent's minimiser (src/brent.cu:43-121) as
// a state machine in device memory, advanced by one thread after every
// objective evaluation (k_ls_step of the CUDA-graph loop, linesearch.cu).
// Kept in a header of its own so any kernel that steps the search shares
// this code.
//
// The arithmetic is the host version's, operation for operation: float
// variables, and the double-precision constants (GOLD 1.618034, GLIMIT 100,
// TINY 1e-20, CGOLD 0.3819660, ZEPS 1e-10) promoting their expressions to
// double exactly where the C++ rules promote them.  Every multiplication is a
// round-to-nearest intrinsic, which the compiler never merges into a fused
// multiply-add, so each operation is rounded on its own -- as in the host
// code, built with -ffp-contract=off -- whatever contraction setting the
// including file is compiled with, and the search visits the same points and
// returns the same minimum bit for bit.
#pragma once

#include "gv_internal.cuh"

namespace gv {
namespace ls {

__device__ __forceinline__ float ls_fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double ls_dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sign_of(float a, float b) { return b >= 0.0 ? fabsf(a) : -fabsf(a); }

enum LsWait {
  kWaitFa = 0,  // bracket: f(ax)
  kWaitFb,      // bracket: f(bx)
  kWaitFc,      // bracket: f(cx)
  kWaitU1,      // bracket: f(u), u between bx and cx
  kWaitU2,      // bracket: f(u), u between cx and ulim
  kWaitShift,   // bracket: f(u), then shift (ax, bx, cx) <- (bx, cx, u)
  kWaitFx,      // Brent: f(x) at the start
  kWaitFu,      // Brent: f(u)
  kDone
};

// Takes f at the point last asked for and advances; returns true when it asks
// for another evaluation (at s.x_req), false when the search is over.
__device__ inline bool ls_advance(LsState& s, float f) {
  const double gold = 1.618034, glimit = 100.0, tiny = 1.0e-20;
  const double cgold = 0.3819660, zeps = 1.0e-10;
  enum { kResume, kShift, kBracketLoop, kBracketDone, kBrentTop } at = kResume;
  for (;;) {
    switch (at) {
      case kResume:
        switch (s.state) {
          case kWaitFa:
            s.fa = f;
            s.x_req = s.bx;
            s.state = kWaitFb;
            return true;
          case kWaitFb: {
            s.fb = f;
            if (s.fb > s.fa) {
              const float t = s.ax;
              s.ax = s.bx;
              s.bx = t;
              const float ft = s.fa;
              s.fa = s.fb;
              s.fb = ft;
            }
            s.cx = (float)(s.bx + ls_dmul(gold, s.bx - s.ax));
            s.x_req = s.cx;
            s.state = kWaitFc;
            return true;
          }
          case kWaitFc:
            s.fc = f;
            at = kBracketLoop;
            break;
          case kWaitU1:
            s.fu = f;
            if (s.fu < s.fc) {
              s.ax = s.bx;
              s.bx = s.u;
              s.fa = s.fb;
              s.fb = s.fu;
              at = kBracketDone;
              break;
            } else if (s.fu > s.fb) {
              s.cx = s.u;
              s.fc = s.fu;
              at = kBracketDone;
              break;
            }
            s.u = (float)(s.cx + ls_dmul(gold, s.cx - s.bx));
            s.x_req = s.u;
            s.state = kWaitShift;
            return true;
          case kWaitU2:
            s.fu = f;
            if (s.fu < s.fc) {
              s.bx = s.cx;
              s.cx = s.u;
              s.u = (float)(s.cx + ls_dmul(gold, s.cx - s.bx));
              s.fb = s.fc;
              s.fc = s.fu;
              s.x_req = s.u;
              s.state = kWaitShift;
              return true;
            }
            at = kShift;
            break;
          case kWaitShift:
            s.fu = f;
            at = kShift;
            break;
          case kWaitFx:
            s.fx = f;
            s.fw = s.fv = s.fx;
            s.it = 1;
            at = kBrentTop;
            break;
          case kWaitFu: {
            s.fu = f;
            const float u = s.u, fu = s.fu;
            if (fu <= s.fx) {
              if (u >= s.x)
                s.a = s.x;
              else
                s.b = s.x;
              s.v = s.w;
              s.w = s.x;
              s.x = u;
              s.fv = s.fw;
              s.fw = s.fx;
              s.fx = fu;
            } else {
              if (u < s.x)
                s.a = u;
              else
                s.b = u;
              if (fu <= s.fw || s.w == s.x) {
                s.v = s.w;
                s.w = u;
                s.fv = s.fw;
                s.fw = fu;
              } else if (fu <= s.fv || s.v == s.x || s.v == s.w) {
                s.v = u;
                s.fv = fu;
              }
            }
            s.it++;
            at = kBrentTop;
            break;
          }
          default:
            return false;
        }
        break;
      case kShift:
        s.ax = s.bx;
        s.bx = s.cx;
        s.cx = s.u;
        s.fa = s.fb;
        s.fb = s.fc;
        s.fc = s.fu;
        at = kBracketLoop;
        break;
      case kBracketLoop: {
        if (!(s.fb > s.fc)) {
          at = kBracketDone;
          break;
        }
        const float r = ls_fmul(s.bx - s.ax, s.fb - s.fc);
        const float q = ls_fmul(s.bx - s.cx, s.fb - s.fa);
        const float aq = fabsf(q - r), atiny = (float)tiny;
        const float den = aq > atiny ? aq : atiny;
        float u = (float)(s.bx - (ls_fmul(s.bx - s.cx, q) - ls_fmul(s.bx - s.ax, r)) /
                                     ls_dmul(2.0, sign_of(den, q - r)));
        const float ulim = (float)(s.bx + ls_dmul(glimit, s.cx - s.bx));
        int wait;
        if (ls_fmul(s.bx - u, u - s.cx) > 0.0) {
          wait = kWaitU1;
        } else if (ls_fmul(s.cx - u, u - ulim) > 0.0) {
          wait = kWaitU2;
        } else if (ls_fmul(u - ulim, ulim - s.cx) >= 0.0) {
          u = ulim;
          wait = kWaitShift;
        } else {
          u = (float)(s.cx + ls_dmul(gold, s.cx - s.bx));
          wait = kWaitShift;
        }
        s.u = u;
        s.x_req = u;
        s.state = wait;
        return true;
      }
      case kBracketDone:
        // brent(ax, bx, cx): the middle point bx starts the search
        s.a = s.ax < s.cx ? s.ax : s.cx;
        s.b = s.ax > s.cx ? s.ax : s.cx;
        s.d = 0.0f;
        s.e = 0.0f;
        s.x = s.w = s.v = s.bx;
        s.x_req = s.x;
        s.state = kWaitFx;
        return true;
      case kBrentTop: {
        if (s.it > 500) {
          s.xmin = s.x;
          s.fret = s.fx;
          s.state = kDone;
          return false;
        }
        const float xm = (float)ls_dmul(0.5, s.a + s.b);
        const float tol1 = (float)(ls_fmul(s.tol, fabsf(s.x)) + zeps);
        const float tol2 = (float)ls_dmul(2.0, tol1);
        if (fabsf(s.x - xm) <= (tol2 - ls_dmul(0.5, s.b - s.a))) {
          s.xmin = s.x;
          s.fret = s.fx;
          s.state = kDone;
          return false;
        }
        if (fabsf(s.e) > tol1) {
          const float r = ls_fmul(s.x - s.w, s.fx - s.fv);
          float q = ls_fmul(s.x - s.v, s.fx - s.fw);
          float pp = ls_fmul(s.x - s.v, q) - ls_fmul(s.x - s.w, r);
          q = (float)ls_dmul(2.0, q - r);
          if (q > 0.0) pp = -pp;
          q = fabsf(q);
          const float etemp = s.e;
          s.e = s.d;
          if (fabsf(pp) >= fabs(ls_dmul(ls_dmul(0.5, q), etemp)) || pp <= ls_fmul(q, s.a - s.x) ||
              pp >= ls_fmul(q, s.b - s.x)) {
            s.e = s.x >= xm ? s.a - s.x : s.b - s.x;
            s.d = (float)ls_dmul(cgold, s.e);
          } else {
            s.d = pp / q;
            const float u = s.x + s.d;
            if (u - s.a < tol2 || s.b - u < tol2) s.d = sign_of(tol1, xm - s.x);
          }
        } else {
          s.e = s.x >= xm ? s.a - s.x : s.b - s.x;
          s.d = (float)ls_dmul(cgold, s.e);
        }
        s.u = fabsf(s.d) >= tol1 ? s.x + s.d : s.x + sign_of(tol1, s.d);
        s.x_req = s.u;
        s.state = kWaitFu;
        return true;
      }
    }
  }
}

// One step of the search after an evaluation, on a state the caller holds:
// f is ObjectiveFunction's calcFunction from the term values in scal (sum of
// lambda_t * value_t in FP64, rounded to float); the search advances to its
// next point (true) or ends (false), also after `cap` evaluations (error 1).
// At the end fret, the evaluation count, the error flag and xmin go to
// scal[kSlotLs..kSlotLs+3].  The term values are read through L2.
__device__ inline bool ls_step_on(LsState& s, double* scal) {
  double fd = 0.0;
  for (int t = 0; t < s.nterms; t++) fd += ls_dmul((double)s.lambda[t], __ldcg(scal + kSlotTerm0 + t));
  s.evals++;
  s.steps++;
  bool more = ls_advance(s, (float)fd);
  if (more && s.steps >= s.cap) {
    more = false;
    s.error = 1;
    s.xmin = s.x_req;
    s.fret = (float)fd;
  }
  if (!more) {
    scal[kSlotLs] = (double)s.fret;
    scal[kSlotLs + 1] = (double)s.evals;
    scal[kSlotLs + 2] = (double)s.error;
    scal[kSlotLs + 3] = (double)s.xmin;
  }
  return more;
}

// The same on the state in global memory, read through L2 (the thread that
// steps may run on a different SM from one evaluation to the next).
__device__ inline bool ls_step(LsState* gs, double* scal) {
  LsState s;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(gs);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s);
    for (int i = 0; i < (int)(sizeof(LsState) / sizeof(uint32_t)); i++) dst[i] = __ldcg(src + i);
  }
  const bool more = ls_step_on(s, scal);
  *gs = s;
  return more;
}

}  // namespace ls
}  // namespace gv
