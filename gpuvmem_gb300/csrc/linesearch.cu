// linmin's line search on the GPU: the bracketing step (src/mnbrak.cu:44-98)
// and Brent's minimiser (src/brent.cu:43-121) as a state machine in device
// memory, advanced by one thread after every objective evaluation.  With the
// evaluation kernels it forms the body of a CUDA-graph WHILE loop
// (optim.cu), so a whole line search is one graph launch with no host
// round trip per evaluation.
//
// The arithmetic is the host version's, operation for operation: float
// variables, the double-precision constants (GOLD 1.618034, GLIMIT 100,
// TINY 1e-20, CGOLD 0.3819660, ZEPS 1e-10) promoting their expressions to
// double exactly where the C++ rules promote them, and this file is
// compiled without FMA contraction (-fmad=false) as the host code is
// (-ffp-contract=off), so the search visits the same points and returns the
// same minimum bit for bit.  The loop ends after `cap` evaluations at the
// latest (the host bracketing loop has no bound; an unbounded decrease along
// the line ends here with an error status instead).
#include "gv_internal.cuh"

namespace gv {
namespace {

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

__device__ __forceinline__ float sign_of(float a, float b) { return b >= 0.0 ? fabsf(a) : -fabsf(a); }

// Takes f at the point last asked for and advances; returns true when it asks
// for another evaluation (at s.x_req), false when the search is over.
__device__ bool ls_advance(LsState& s, float f) {
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
            s.cx = (float)(s.bx + gold * (s.bx - s.ax));
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
            s.u = (float)(s.cx + gold * (s.cx - s.bx));
            s.x_req = s.u;
            s.state = kWaitShift;
            return true;
          case kWaitU2:
            s.fu = f;
            if (s.fu < s.fc) {
              s.bx = s.cx;
              s.cx = s.u;
              s.u = (float)(s.cx + gold * (s.cx - s.bx));
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
        const float r = (s.bx - s.ax) * (s.fb - s.fc);
        const float q = (s.bx - s.cx) * (s.fb - s.fa);
        const float aq = fabsf(q - r), atiny = (float)tiny;
        const float den = aq > atiny ? aq : atiny;
        float u = (float)(s.bx - ((s.bx - s.cx) * q - (s.bx - s.ax) * r) /
                                     (2.0 * sign_of(den, q - r)));
        const float ulim = (float)(s.bx + glimit * (s.cx - s.bx));
        int wait;
        if ((s.bx - u) * (u - s.cx) > 0.0) {
          wait = kWaitU1;
        } else if ((s.cx - u) * (u - ulim) > 0.0) {
          wait = kWaitU2;
        } else if ((u - ulim) * (ulim - s.cx) >= 0.0) {
          u = ulim;
          wait = kWaitShift;
        } else {
          u = (float)(s.cx + gold * (s.cx - s.bx));
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
        const float xm = (float)(0.5 * (s.a + s.b));
        const float tol1 = (float)(s.tol * fabsf(s.x) + zeps);
        const float tol2 = (float)(2.0 * tol1);
        if (fabsf(s.x - xm) <= (tol2 - 0.5 * (s.b - s.a))) {
          s.xmin = s.x;
          s.fret = s.fx;
          s.state = kDone;
          return false;
        }
        if (fabsf(s.e) > tol1) {
          const float r = (s.x - s.w) * (s.fx - s.fv);
          float q = (s.x - s.v) * (s.fx - s.fw);
          float pp = (s.x - s.v) * q - (s.x - s.w) * r;
          q = (float)(2.0 * (q - r));
          if (q > 0.0) pp = -pp;
          q = fabsf(q);
          const float etemp = s.e;
          s.e = s.d;
          if (fabsf(pp) >= fabs(0.5 * q * etemp) || pp <= q * (s.a - s.x) ||
              pp >= q * (s.b - s.x)) {
            s.e = s.x >= xm ? s.a - s.x : s.b - s.x;
            s.d = (float)(cgold * s.e);
          } else {
            s.d = pp / q;
            const float u = s.x + s.d;
            if (u - s.a < tol2 || s.b - u < tol2) s.d = sign_of(tol1, xm - s.x);
          }
        } else {
          s.e = s.x >= xm ? s.a - s.x : s.b - s.x;
          s.d = (float)(cgold * s.e);
        }
        s.u = fabsf(s.d) >= tol1 ? s.x + s.d : s.x + sign_of(tol1, s.d);
        s.x_req = s.u;
        s.state = kWaitFu;
        return true;
      }
    }
  }
}

__global__ void k_ls_begin(LsState* s, LsTerms terms, float tol, int cap) {
  if (threadIdx.x != 0) return;
  s->state = kWaitFa;
  s->evals = 0;
  s->steps = 0;
  s->it = 0;
  s->error = 0;
  s->cap = cap;
  s->tol = tol;
  s->nterms = terms.nterms;
  for (int t = 0; t < kMaxTerms; t++) s->lambda[t] = terms.lambda[t];
  // linmin: ax = 0, xx = 1 (src/linmin.cu:78-80)
  s->ax = 0.0f;
  s->bx = 1.0f;
  s->x_req = s->ax;
  s->xmin = 0.0f;
  s->fret = 0.0f;
}

__global__ void k_ls_step(LsState* s, double* scal, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0) return;
  // ObjectiveFunction::calcFunction as a float: sum of lambda * term value
  double fd = 0.0;
  for (int t = 0; t < s->nterms; t++) fd += (double)s->lambda[t] * scal[kSlotTerm0 + t];
  s->evals++;
  s->steps++;
  bool more = ls_advance(*s, (float)fd);
  if (more && s->steps >= s->cap) {
    more = false;
    s->error = 1;
    s->xmin = s->x_req;
    s->fret = (float)fd;
  }
  if (!more) {
    scal[kSlotLs] = (double)s->fret;
    scal[kSlotLs + 1] = (double)s->evals;
    scal[kSlotLs + 2] = (double)s->error;
    scal[kSlotLs + 3] = (double)s->xmin;
  }
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

}  // namespace

gv_status ls_begin_launch(cudaStream_t st, LsState* s, LsTerms terms, float tol, int cap) {
  k_ls_begin<<<1, 32, 0, st>>>(s, terms, tol, cap);
  GV_LAUNCH("k_ls_begin");
  return GV_OK;
}

gv_status ls_step_launch(cudaStream_t st, LsState* s, double* scal, cudaGraphConditionalHandle h) {
  k_ls_step<<<1, 32, 0, st>>>(s, scal, h);
  GV_LAUNCH("k_ls_step");
  return GV_OK;
}

}  // namespace gv
