// k_transport.cuh - persistent Monte Carlo packet-transport kernel.
//
// GB300 design: one thread owns one packet history; a warp keeps all 32 lanes
// busy by refilling idle lanes from a device work queue with one
// warp-aggregated atomic per refill.  Each loop iteration advances every lane
// by one event (an emission, or one cell step of pathSegment), so the lanes of
// a warp stay on the same code path.  Packet geometry and optical depth run in
// the template precision R (float: the production path; double: the plain
// FP64 path); the mean-intensity estimator J_nu is accumulated with FP64
// atomics into the Fortran-layout array Jste[nu][cell], compensated: each
// atomic's exact rounding error (TwoSum of the value it returned and the
// deposit) goes to a second array Jlo, folded in after the launch, so the
// result is the correctly rounded sum of the deposits whatever their order.  The source spectrum
// CDF, the frequency mesh and the axes are staged in shared memory.
//
// Physics follows the reference routine by routine (single mother grid, no
// plane-parallel illumination):
//   energyPacketDriver/energyPacketRun   source/photon_mod.f90:28-741
//   initPhotonPacket / getNu2            source/photon_mod.f90:744-972
//   newPhotonPacket                      source/photon_mod.f90:976-1756
//   pathSegment                          source/photon_mod.f90:1758-4085
//   comptonScatter                       source/photon_mod.f90:6805-6848
// Packet k of a call (global id counter_base + k) draws its uniforms from its
// own Philox4x32-10 stream, so a history does not depend on scheduling.
// Jste(0,:), the dump row the reference fills for inactive cells and never
// reads, is not accumulated.
#pragma once
#include "k_transport_launch.h"
#include "mcx_device.cuh"
#include "mcx_fmath.h"

namespace mcx {

enum : int { PT_STELLAR = 0, PT_DIFFUSE = 1, PT_DUSTEMI = 2 };
enum : int { ST_IDLE = 0, ST_EMIT = 1, ST_STEP = 2, ST_DONE = 3, ST_ESCAPE = 4 };

constexpr int kSafeLimit = 500000;        // pathSegment (source/photon_mod.f90:1873-1878)
constexpr int kSafeLimitPlane = 5000;     // the same, plane-parallel ionisation
constexpr int kRecursionLimit = 100000;   // recursionLimit (source/constants_mod.f90:70)

template <typename R> struct RMath;
template <> struct RMath<float> {
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float log_(float x) { return logf(x); }
  static __device__ __forceinline__ float cos_(float x) { return cosf(x); }
  static __device__ __forceinline__ float sin_(float x) { return sinf(x); }
  static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
  static __device__ __forceinline__ float min_(float a, float b) { return fminf(a, b); }
  // the step's quotients: reciprocal-approximation division (2 ulp; operands far below 2^126)
  static __device__ __forceinline__ float div_(float a, float b) { return __fdividef(a, b); }
};
// the plain FP64 path: log, cos and sin from the portable routines the oracle
// uses too (mcx_fmath.h), so that both draw the same packet histories
template <> struct RMath<double> {
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double log_(double x) { return mcx_fm_log(x); }
  static __device__ __forceinline__ double cos_(double x) { return mcx_fm_cos(x); }
  static __device__ __forceinline__ double sin_(double x) { return mcx_fm_sin(x); }
  static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
  static __device__ __forceinline__ double min_(double a, double b) { return fmin(a, b); }
  static __device__ __forceinline__ double div_(double a, double b) { return a / b; }
};

// t cos(a) and t sin(a), out of line: the accurate sine and cosine are long,
// and inlined at each direction draw they would crowd the transport loop out
// of the instruction cache.
template <typename R>
struct CosSin { R c, s; };

template <typename R>
__device__ __noinline__ CosSin<R> scaledCosSin(R t, R a) {
  using M = RMath<R>;
  return CosSin<R>{t * M::cos_(a), t * M::sin_(a)};
}

// The isotropic direction initPhotonPacket draws from the uniforms r1, r2
// (source/photon_mod.f90:858-878): w = 2 r1 - 1, t = sqrt(1 - w^2),
// phi = pi (2 r2 - 1), (t cos phi, t sin phi, w).
template <typename R>
struct Dir3 { R x, y, z; };

template <typename R>
__device__ __forceinline__ Dir3<R> isoDirection(R r1, R r2) {
  using M = RMath<R>;
  const R w = R(2) * r1 - R(1);
  const R t = M::sqrt_(R(1) - w * w);
  const R ang = R(3.141592654) * (R(2) * r2 - R(1));
  const CosSin<R> cs = scaledCosSin<R>(t, ang);
  return Dir3<R>{cs.c, cs.s, w};
}

// One lane's share of a warp history's CDF search (see warpCdfIssue).
struct WarpCdf {
  float v;          // this lane's segment end
  int seg, segs;    // segment length (a multiple of 32) and segments probed
};

template <typename R>
struct Packet {
  using Real = R;
  static constexpr bool kWarp = false;   // one lane per history
  R x, y, z, vx, vy, vz;
  R ex, ey, ez;     // the direction the current path segment started with (the escape tally's)
  R nu, absTau, passProb;
  int xP, yP, zP, nuP, origin;
  int type, lgStellar, nEmit, nStep;
  PacketRng rng;
};

// A history run by a whole warp (the trapped-packet kernel): every lane holds
// the same state and executes the same scalar arithmetic, so every lane
// computes the same values; the lanes split only the data-parallel parts.
// Here the Philox stream: lane l keeps block blk0 + l (draws 4 (blk0 + l) ..
// 4 (blk0 + l) + 3), so one refill covers the next 128 draws and a draw is a
// select and a shuffle.  At a refill each lane also evaluates, for each of its
// four positions i, what a history drawing there would compute: the isotropic
// direction from draws i and i + 1 and -ln(1 - u_i) (a path's optical depth),
// so that the history's chain of events takes them with a shuffle instead of a
// square root, a sine, a cosine and a logarithm.  Lookups go by the draw index
// the history has reached, so any sequence of draws finds its own values; the
// values are those of the same expressions, bit for bit.
template <typename R>
struct WarpRng {
  uint32_t k0, k1, p0, p1;
  uint32_t k;              // draws taken so far
  uint32_t blk0;           // first Philox block held by the warp
  uint32_t b0, b1, b2, b3; // this lane's block, blk0 + lane
  R dx0, dx1, dx2, dx3, dy0, dy1, dy2, dy3, dz0, dz1, dz2, dz3;   // direction starting at position c
  R nl0, nl1, nl2, nl3;                                           // -ln(1 - u) at position c
  __device__ __forceinline__ void fill(uint32_t first) {
    using M = RMath<R>;
    blk0 = first;
    const uint4 b = philoxBlock(p0, p1, first + (threadIdx.x & 31u), k0, k1);
    b0 = b.x; b1 = b.y; b2 = b.z; b3 = b.w;
    // the next lane's first draw completes the direction starting at position 3
    // (lane 31's lies beyond the window; it is never looked up)
    const uint32_t after = __shfl_down_sync(0xffffffffu, b0, 1);
    const R u0 = uniformFrom<R>(b0), u1 = uniformFrom<R>(b1), u2 = uniformFrom<R>(b2), u3 = uniformFrom<R>(b3);
    const R u4 = uniformFrom<R>(after);
    Dir3<R> d;
    d = isoDirection<R>(u0, u1); dx0 = d.x; dy0 = d.y; dz0 = d.z;
    d = isoDirection<R>(u1, u2); dx1 = d.x; dy1 = d.y; dz1 = d.z;
    d = isoDirection<R>(u2, u3); dx2 = d.x; dy2 = d.y; dz2 = d.z;
    d = isoDirection<R>(u3, u4); dx3 = d.x; dy3 = d.y; dz3 = d.z;
    nl0 = -M::log_(R(1) - u0); nl1 = -M::log_(R(1) - u1);
    nl2 = -M::log_(R(1) - u2); nl3 = -M::log_(R(1) - u3);
  }
  __device__ __forceinline__ void start(const PacketRng& r) {
    k0 = r.k0; k1 = r.k1; p0 = r.p0; p1 = r.p1; k = r.k;
    fill(k >> 2);
  }
  template <typename T>
  static __device__ __forceinline__ T pick(uint32_t c, T a0, T a1, T a2, T a3) {
    return c == 0u ? a0 : (c == 1u ? a1 : (c == 2u ? a2 : a3));
  }
  // the lane holding position k, refilling the window first if k has left it
  __device__ __forceinline__ int lane() {
    if ((k >> 2) - blk0 >= 32u) fill(k >> 2);
    return (int)((k >> 2) - blk0);
  }
  __device__ __forceinline__ uint32_t next() {
    const int src = lane();
    const uint32_t c = k & 3u;
    ++k;
    return __shfl_sync(0xffffffffu, pick(c, b0, b1, b2, b3), src);
  }
  // -ln(1 - u) of the next draw
  __device__ __forceinline__ R negLog1m() {
    const int src = lane();
    const uint32_t c = k & 3u;
    ++k;
    return __shfl_sync(0xffffffffu, pick(c, nl0, nl1, nl2, nl3), src);
  }
  // the isotropic direction from the next two draws
  __device__ __forceinline__ Dir3<R> direction() {
    const int src = lane();
    const uint32_t c = k & 3u;
    if (src == 31 && c == 3u) {   // its second draw is in the next window
      const R r1 = uniformFrom<R>(next());
      const R r2 = uniformFrom<R>(next());
      return isoDirection<R>(r1, r2);
    }
    k += 2;
    const unsigned FULL = 0xffffffffu;
    return Dir3<R>{__shfl_sync(FULL, pick(c, dx0, dx1, dx2, dx3), src),
                   __shfl_sync(FULL, pick(c, dy0, dy1, dy2, dy3), src),
                   __shfl_sync(FULL, pick(c, dz0, dz1, dz2, dz3), src)};
  }
};

template <typename R>
struct WarpPacket {
  using Real = R;
  static constexpr bool kWarp = true;
  R x, y, z, vx, vy, vz;
  R ex, ey, ez;
  R nu, absTau, passProb;
  int xP, yP, zP, nuP, origin;
  int type, lgStellar, nEmit, nStep;
  WarpRng<R> rng;
  int2 cdfShape;     // warpCdfShape(nbins), computed once per launch
  __device__ __forceinline__ void from(const Packet<R>& a) {
    x = a.x; y = a.y; z = a.z; vx = a.vx; vy = a.vy; vz = a.vz;
    ex = a.ex; ey = a.ey; ez = a.ez;
    nu = a.nu; absTau = a.absTau; passProb = a.passProb;
    xP = a.xP; yP = a.yP; zP = a.zP; nuP = a.nuP; origin = a.origin;
    type = a.type; lgStellar = a.lgStellar; nEmit = a.nEmit; nStep = a.nStep;
    rng.start(a.rng);
  }
};

// Whether this lane performs the history's side effects (atomics): every lane
// of a one-lane history, lane 0 of a warp history.
template <typename P>
__device__ __forceinline__ bool effectLane() { return !P::kWarp || (threadIdx.x & 31u) == 0u; }

// Shared memory of a transport block after its tables: each thread's packet
// state (one Packet per thread; its address goes to the out-of-line emission
// code, so it cannot live in registers, and shared memory keeps it on chip).
__host__ __device__ constexpr size_t packetStateOffset(size_t tableBytes) { return (tableBytes + 15) / 16 * 16; }
template <typename R>
__host__ __device__ constexpr size_t packetStateBytes(int threads) { return (size_t)threads * sizeof(Packet<R>); }

struct LocalCounters {
  unsigned long long crossings = 0, interactions = 0, absorptions = 0, scatterings = 0;
  unsigned long long escaped = 0, lineEscapes = 0, trapped = 0, emissions = 0, errors = 0;
  double qPhot = 0.;
};

template <typename R>
struct TransportShared {
  const float* nu;           // frequency mesh (shared memory)
};

// The grid a packet travels in, read through accessors so that one emit /
// step code serves both kernels: OneGrid<plane> reads the context's single grid from
// the kernel parameters (axes and source CDF staged in shared memory);
// NebulaGeo holds, in registers, the nebula of a batch that the packet belongs
// to (axes, active map and CDF slices of the concatenated batch arrays; the
// active map holds batch-wide cell ids).
template <bool kPlane>
struct OneGrid {
  const DevGrid& g;
  const float* sX; const float* sY; const float* sZ; const float* sCdf;
  __device__ __forceinline__ int nx() const { return g.nx; }
  __device__ __forceinline__ int ny() const { return g.ny; }
  __device__ __forceinline__ int nz() const { return g.nz; }
  __device__ __forceinline__ int symmetric() const { return g.symmetric; }
  __device__ __forceinline__ float rOut() const { return g.rOut; }
  __device__ __forceinline__ const float* X() const { return sX; }
  __device__ __forceinline__ const float* Y() const { return sY; }
  __device__ __forceinline__ const float* Z() const { return sZ; }
  __device__ __forceinline__ const int32_t* active() const { return g.active; }
  __device__ __forceinline__ bool activeFull() const { return g.activeFull != 0; }
  // fixed per instantiation: the kernels are built with and without the
  // plane-parallel source, so that other grids carry none of its code
  __device__ __forceinline__ constexpr bool plane() const { return kPlane; }
  __device__ __forceinline__ const float* cdf() const { return sCdf; }
  __device__ __forceinline__ int starIdx(int d) const { return g.starIdx[d]; }
  __device__ __forceinline__ float starPos(int d) const { return g.starPos[d]; }
};

struct NebulaGeo {
  int nx_, ny_, nz_, symmetric_;
  float rOut_;
  const float* X_; const float* Y_; const float* Z_;
  const int32_t* active_;
  const float* cdf_;
  int starIdx_[3];
  float starPos_[3];
  __device__ __forceinline__ int nx() const { return nx_; }
  __device__ __forceinline__ int ny() const { return ny_; }
  __device__ __forceinline__ int nz() const { return nz_; }
  __device__ __forceinline__ int symmetric() const { return symmetric_; }
  __device__ __forceinline__ float rOut() const { return rOut_; }
  __device__ __forceinline__ const float* X() const { return X_; }
  __device__ __forceinline__ const float* Y() const { return Y_; }
  __device__ __forceinline__ const float* Z() const { return Z_; }
  __device__ __forceinline__ const int32_t* active() const { return active_; }
  __device__ __forceinline__ bool activeFull() const { return false; }
  __device__ __forceinline__ constexpr bool plane() const { return false; }
  __device__ __forceinline__ const float* cdf() const { return cdf_; }
  __device__ __forceinline__ int starIdx(int d) const { return starIdx_[d]; }
  __device__ __forceinline__ float starPos(int d) const { return starPos_[d]; }
};

template <typename Geo>
__device__ __forceinline__ int activeAt(const Geo& q, int i, int j, int k) {
  if (q.activeFull()) return ((i - 1) * q.ny() + (j - 1)) * q.nz() + k;
  return __ldg(q.active() + (size_t)(i - 1) + (size_t)q.nx() * ((size_t)(j - 1) + (size_t)q.ny() * (size_t)(k - 1)));
}

// Packets re-emitted this many times are taken to be trapped in optically thick
// cells: their lane runs on, often alone in its warp, long after the others
// are done, so each dependent global load of its events is paid in full.  For
// these lanes the emission prefetches the cell's whole CDF row into L1 before
// the bisection, and the step prefetches the scattering inputs with the
// opacity.  Prefetches change no value read, only when it arrives.
constexpr int kTrappedHint = 8;

__device__ __forceinline__ void prefetchL1(const void* a) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
}

// every 128-byte line of the n floats at row
__device__ __forceinline__ void prefetchRowL1(const float* row, int n) {
  for (int i = 0; i < n; i += 32) prefetchL1(row + i);
  prefetchL1(row + (n - 1));
}

// getNu2 on a monotone CDF: the reference's linear scan "last i with u >= cdf(i)"
// equals the count of leading entries <= u, found here by bisection.
template <typename R>
__device__ __forceinline__ int sampleCDF(const float* cdf, int len, int nbins, R u) {
  int lo = 0, hi = len < nbins ? len : nbins;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (u >= (R)cdf[mid]) lo = mid + 1; else hi = mid;
  }
  int nuP = lo < 1 ? 1 : lo;
  if (nuP < nbins) ++nuP;
  return nuP;
}

// sampleCDF's count for a warp history, the 32 lanes comparing in parallel:
// first the last entry of each of up to 32 segments (issued by warpCdfIssue
// as soon as the row is known, before u is drawn), then the entries of the
// one segment that holds the answer.  On a monotone row the count of entries
// <= u does not depend on the order of the comparisons, so the result equals
// the bisection's.
// the segmentation of an m-entry row (fixed for a launch)
__device__ __forceinline__ int2 warpCdfShape(int m) {
  const int seg = 32 * ((m + 1023) / 1024);
  return make_int2(seg, m / seg);
}

__device__ __forceinline__ void warpCdfIssue(WarpCdf& c, const float* __restrict__ row, int2 shape) {
  const int lane = threadIdx.x & 31;
  c.seg = shape.x;
  c.segs = shape.y;
  c.v = lane < c.segs ? __ldg(row + (size_t)(lane + 1) * c.seg - 1) : 0.f;
}

template <typename R>
__device__ __forceinline__ int warpCdfFinish(const WarpCdf& c, const float* __restrict__ row, int m, int nbins, R u) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int s = __popc(__ballot_sync(FULL, lane < c.segs && u >= (R)c.v));
  const int base = s * c.seg;
  const int end = base + c.seg < m ? base + c.seg : m;
  int lo = base;
  for (int b = base; b < end; b += 32) {
    const bool in = b + lane < end;
    const float w = in ? __ldg(row + b + lane) : 0.f;
    lo += __popc(__ballot_sync(FULL, in && u >= (R)w));
  }
  int nuP = lo < 1 ? 1 : lo;
  if (nuP < nbins) ++nuP;
  return nuP;
}

template <typename P>
__device__ __forceinline__ typename P::Real draw(P& p) { return uniformFrom<typename P::Real>(p.rng.next()); }

// a path's optical depth to the next interaction, -ln(1 - u)
template <typename P>
__device__ __forceinline__ typename P::Real drawPassProb(P& p) {
  using R = typename P::Real;
  if constexpr (P::kWarp) return p.rng.negLog1m();
  else return -RMath<R>::log_(R(1) - draw(p));
}

// locate (source/interpolation_mod.f90:49-106) on the frequency mesh or an axis
template <typename R>
__device__ __forceinline__ int locateNu(const float* xa, int n, R x) {
  if (x > (R)xa[n - 1]) return n;
  if (x < (R)xa[0]) return 0;
  int jlow = 0, jup = n + 1;
  for (int it = 0; it < 64; ++it) {
    if (jup - jlow < 1) break;
    int jm = (jup + jlow) >> 1;
    R v = (R)xa[jm - 1];
    if (v == x) return jm;
    if (x > v) { if (jlow == jm) break; jlow = jm; } else jup = jm;
  }
  return jlow;
}

// initPhotonPacket (source/photon_mod.f90:744-896): position, frequency, an
// isotropic direction (re-drawn while a component is exactly zero) and the
// octant fold for stellar packets.
template <typename R, typename Geo, typename P>
__device__ __forceinline__ void initPacket(const Geo& q, const TransportShared<R>& sh, P& p, int nuP,
                                           bool line, bool stellar, int xP, int yP, int zP) {
  using M = RMath<R>;
  p.nuP = nuP;
  p.lgStellar = stellar;
  p.nu = line ? R(0) : (R)sh.nu[nuP - 1];
  if (stellar && q.plane()) {
    // the ionising plane (source/photon_mod.f90:795-856): born on y = 0 at a
    // uniform (x, z) within the axes' span, in the cell whose walls bracket it,
    // moving along +y
    const float* X = q.X(); const float* Z = q.Z();
    const int nx = q.nx(), nz = q.nz();
    R rnd = R(1) - draw(p);
    p.x = (R)X[0] + rnd * ((R)X[nx - 1] - (R)X[0]);
    xP = locateNu<R>(X, nx, p.x);
    if (xP < nx && xP > 0 && p.x >= ((R)X[xP - 1] + (R)X[xP]) / R(2)) xP = xP + 1;
    p.y = R(0);
    yP = 1;
    rnd = R(1) - draw(p);
    p.z = (R)Z[0] + rnd * ((R)Z[nz - 1] - (R)Z[0]);
    zP = locateNu<R>(Z, nz, p.z);
    if (zP < nz && zP > 0 && p.z >= ((R)Z[zP - 1] + (R)Z[zP]) / R(2)) zP = zP + 1;
    if (xP < 1) xP = 1;
    if (zP < 1) zP = 1;
    p.vx = R(0); p.vy = R(1); p.vz = R(0);
  } else {
    for (int rep = 0; rep < 1000000; ++rep) {
      Dir3<R> d;
      if constexpr (P::kWarp) {
        d = p.rng.direction();
      } else {
        const R r1 = draw(p);
        const R r2 = draw(p);
        d = isoDirection<R>(r1, r2);
      }
      p.vx = d.x; p.vy = d.y; p.vz = d.z;
      if (p.vx != R(0) && p.vy != R(0) && p.vz != R(0)) break;
    }
    if (q.symmetric() && stellar) {
      if (p.vx < R(0)) p.vx = -p.vx;
      if (p.vy < R(0)) p.vy = -p.vy;
      if (p.vz < R(0)) p.vz = -p.vz;
    }
  }
  p.xP = xP; p.yP = yP; p.zP = zP;
  p.ex = p.vx; p.ey = p.vy; p.ez = p.vz;
  p.origin = (xP > 0 && yP > 0 && zP > 0) ? activeAt(q, xP, yP, zP) : 0;
}

// The escape tally (e.g. source/photon_mod.f90:2293-2378): plane 0 of
// escapedPackets always; with viewing angles also plane k when the direction's
// (theta, phi) bin belongs to view k, where theta bins cover [0, pi] in 20 and
// phi bins [0, 2 pi) in totAngleBinsPhi, phi = atan(vy / vx) truncated toward
// zero and taken as 0 for vx < 1e-35 (the reference's own binning: every
// packet leaving with vx <= 0 lands in phi bin 1, and since atan spans
// (-pi/2, pi/2) the bins between pi/2 and 3 pi/2 receive nothing).  Directions in no view's
// bins have viewPointPtheta = viewPointPphi = 0, which the reference's test
// counts as a match of view 0, adding deltaE to plane 0 a second time; both
// are reproduced.
// The (theta, phi) bins of a direction, out of line (acos and atan are long
// and run once per escaping packet).
template <typename R>
__device__ __noinline__ int2 viewBins(R vx, R vy, R vz, int totPhi) {
  const R dTheta = R(3.141592654) / R(20);
  const R dPhi = (R(2) * R(3.141592654)) / (R)totPhi;
  int idirT = (int)(acos(vz) / dTheta) + 1;
  if (idirT > 20) idirT = 20;
  if (idirT < 1) idirT = 1;
  int idirP = vx < R(1.e-35) ? 0 : (int)(atan(vy / vx) / dPhi);
  if (idirP < 0) idirP = totPhi + idirP;
  idirP = idirP + 1;
  if (idirP > totPhi) idirP = totPhi;
  return make_int2(idirT, idirP);
}

template <typename R, typename P>
__device__ __forceinline__ void escapeTally(const DevGrid& g, const DevTransportOut& out, const P& p,
                                            double deltaE, LocalCounters& lc) {
  ++lc.escaped;
  if (!effectLane<P>()) return;
  const size_t plane = ((size_t)g.nCells + 1) * ((size_t)g.nbins + 1);
  const size_t at = (size_t)p.origin + ((size_t)g.nCells + 1) * (size_t)p.nuP;
  if (g.nAngle > 0) {
    // the direction the segment started with: pathSegment tallies
    // enPacket%direction, not the reflected vHat (source/photon_mod.f90:1837)
    const int2 bins = viewBins<R>(p.ex, p.ey, p.ez, g.totPhi);
    const int idirT = bins.x, idirP = bins.y;
    const int k = g.viewPTheta[idirT];
    if ((g.totPhi > 1 && k == g.viewPPhi[idirP]) || (g.totPhi == 1 && k > 0))
      atomicAdd(out.escaped + plane * (size_t)k + at, deltaE);
  }
  atomicAdd(out.escaped + at, deltaE);
}

// A J deposit whose rounding error is still to be added to Jlo.  The FP64
// atomic returns the value it added to; that return is consumed one deposit
// later (or when the lane goes idle), so the wait for it hides behind the
// packet's next step instead of stalling this one.
struct PendingJ {
  double old, v;
  size_t idx;
  bool on;
};

// The exact rounding error of old + v by Fast2Sum (Dekker): with |a| >= |b|,
// b - ((a + b) - a) is exact, three dependent operations where TwoSum takes
// five; the error of a rounded sum is unique, so it is TwoSum's value.  Added
// without a test for zero (adding zero leaves the entry as it is).
__device__ __forceinline__ void flushJ(const DevTransportOut& out, PendingJ& pj) {
  if (pj.on) {
    const double s = pj.old + pj.v;
    const bool ord = fabs(pj.old) >= fabs(pj.v);
    const double big = ord ? pj.old : pj.v, small = ord ? pj.v : pj.old;
    atomicAdd(out.jlo + pj.idx, small - (s - big));
    pj.on = false;
  }
}

template <typename R, bool kWarp>
__device__ __forceinline__ void deposit(const DevGrid& g, const DevTransportOut& out, int cell, int nuP, R dl,
                                        R dV, R deltaE, R costheta, PendingJ& pj) {
  if (cell <= 0 || (kWarp && (threadIdx.x & 31u) != 0u)) return;
  size_t idx = (size_t)cell + ((size_t)g.nCells + 1) * (size_t)(nuP - 1);
  const double v = (double)RMath<R>::div_(dl * deltaE, dV);
  if (out.jlo) {
    flushJ(out, pj);
    pj.old = atomicAdd(out.jste + idx, v);
    pj.v = v;
    pj.idx = idx;
    pj.on = true;
  } else {
    atomicAdd(out.jste + idx, v);
  }
  if (out.hEst) atomicAdd(out.hEst + idx, (double)((dl * deltaE) * costheta / dV));
}

// comptonScatter (source/photon_mod.f90:6805-6848)
template <typename R, typename P>
__device__ __forceinline__ void comptonScatter(const DevGrid& g, const TransportShared<R>& sh, P& p) {
  using M = RMath<R>;
  const float* row = g.KNcdfT + (size_t)(p.nuP - 1) * 180;
  int th = sampleCDF<R>(row, 180, g.nbins, draw(p));
  R newTheta = (R)th * R(3.141592654) / R(180);
  R u = draw(p);
  R w = R(2) * u - R(1);
  R t = M::sqrt_(R(1) - w * w);
  const CosSin<R> cs = scaledCosSin<R>(t, newTheta);
  p.vx = cs.c;
  p.vy = cs.s;
  p.vz = w;
  p.ex = p.vx; p.ey = p.vy; p.ez = p.vz;
  int thc = th > 180 ? 180 : th;
  R newNu = p.nu * (R)__ldg(g.PcompT + (size_t)(p.nuP - 1) * 180 + (thc - 1));
  int newNuP = locateNu<R>(sh.nu, g.nbins, newNu);
  if (newNuP < 1) newNuP = 1;
  p.nu = newNu;
  p.nuP = newNuP;
}

// Volume of cell `cell` in the geometry precision.
template <typename R> __device__ __forceinline__ R cellVolume(const DevGrid& g, int cell);
template <> __device__ __forceinline__ float cellVolume<float>(const DevGrid& g, int cell) { return __ldg(g.volF + cell); }
template <> __device__ __forceinline__ double cellVolume<double>(const DevGrid& g, int cell) { return __ldg(g.volD + cell); }

// energyPacketRun + newPhotonPacket: create the packet of history step p.type
// at (p.x,p.y,p.z; p.xP,p.yP,p.zP).  Returns the next state.  Kept out of line:
// with the step code inlined beside it the loop body overflows the
// instruction cache (measured: 11.9 -> 9.5 ms for 1e7 packets at 41^3).
// For a warp history (P::kWarp) the re-emission CDF search is the warp's,
// its first round issued before the line draw; the same draws, the same result.
template <typename R, typename Geo, typename P>
__device__ __forceinline__ int emitBody(const DevGrid& g, const Geo& q, const DevTransportIn& in, const DevTransportOut& out,
                                        const TransportShared<R>& sh, P& p, double deltaE, LocalCounters& lc) {
  using M = RMath<R>;
  if (p.nEmit >= kRecursionLimit) { ++lc.trapped; return ST_IDLE; }
  ++p.nEmit;
  bool line = false;
  const bool stellar = p.type == PT_STELLAR;
  // the frequency first, then one initPacket for every kind of emission (one
  // copy of the direction code keeps the loop within the instruction cache)
  int nuP = 0, ix = p.xP, iy = p.yP, iz = p.zP;
  if (stellar) {
    nuP = sampleCDF<R>(q.cdf(), g.nbins, g.nbins, draw(p));
    ++lc.emissions;
    p.x = (R)q.starPos(0); p.y = (R)q.starPos(1); p.z = (R)q.starPos(2);
    ix = q.starIdx(0); iy = q.starIdx(1); iz = q.starIdx(2);
  } else {
    if (p.xP < 1 || p.xP > q.nx() || p.yP < 1 || p.yP > q.ny() || p.zP < 1 || p.zP > q.nz()) { ++lc.errors; return ST_IDLE; }
    int cell = activeAt(q, p.xP, p.yP, p.zP);
    if (cell <= 0) { ++lc.errors; return ST_IDLE; }
    const float* cdfTab = p.type == PT_DIFFUSE ? in.recCDFT : in.dustCDFT;
    const float* row = cdfTab ? cdfTab + (size_t)cell * g.nbins : nullptr;
    WarpCdf wc;
    if constexpr (P::kWarp) { if (row) warpCdfIssue(wc, row, p.cdfShape); }
    else if (p.nEmit > kTrappedHint && row) prefetchRowL1(row, g.nbins);
    auto sample = [&](R u) {
      if constexpr (P::kWarp) return warpCdfFinish<R>(wc, row, g.nbins, g.nbins, u);
      else return sampleCDF<R>(row, g.nbins, g.nbins, u);
    };
    if (p.type == PT_DIFFUSE) {
      R rnd = R(1) - draw(p);
      if (rnd <= (R)__ldg(in.totalLines + cell)) {
        line = true;
      } else {
        nuP = sample(draw(p));
        ++lc.emissions;
      }
    } else {
      nuP = sample(draw(p));
      ++lc.emissions;
    }
  }
  initPacket<R>(q, sh, p, nuP, line, stellar, ix, iy, iz);
  if (stellar && p.nu >= R(1)) lc.qPhot += deltaE / (2.1799153e-11 * (double)p.nu);
  if (line) {
    ++lc.lineEscapes;
    if (p.nEmit >= kRecursionLimit) ++lc.trapped;
    return ST_IDLE;
  }
  if (!g.lgDust && p.nu < (R)g.ionEdge1) {
    escapeTally<R>(g, out, p, deltaE, lc);
    if (p.nEmit >= kRecursionLimit) ++lc.trapped;
    return ST_IDLE;
  }
  // pathSegment entry (source/photon_mod.f90:1813-1878)
  if (p.xP <= 0 || p.xP > q.nx() || p.yP <= 0 || p.yP > q.ny() || p.zP <= 0 || p.zP > q.nz()) { ++lc.errors; return ST_IDLE; }
  p.absTau = R(0);
  p.passProb = drawPassProb(p);
  p.nStep = 0;
  return ST_STEP;
}

template <typename R, typename Geo>
__device__ __noinline__ int emitPacket(const DevGrid& g, const Geo& q, const DevTransportIn& in, const DevTransportOut& out,
                                       const TransportShared<R>& sh, Packet<R>& p, double deltaE, LocalCounters& lc) {
  return emitBody<R, Geo>(g, q, in, out, sh, p, deltaE, lc);
}

// One axis of a step's wall geometry (pathSegment, source/photon_mod.f90:
// 1882-2084), written without branches so that the three axes' arithmetic
// interleaves; every value is the reference's expression, so the results are
// those of its branch-by-branch form.  A holds the axis (cell centres) as
// A[0] .. A[n-1], the reference's A(1) .. A(n); a is a 1-based cell index.
template <typename R>
struct AxisVals { R m2, m1, c0, p1, p2, first, last; };   // A(a-2) .. A(a+2) (clamped), A(1), A(n)

template <typename R>
__device__ __forceinline__ AxisVals<R> axisLoad(const float* A, int n, int a) {
  auto at = [&](int i) { i = i < 1 ? 1 : (i > n ? n : i); return (R)A[i - 1]; };
  return AxisVals<R>{at(a - 2), at(a - 1), at(a), at(a + 1), at(a + 2), (R)A[0], (R)A[n - 1]};
}

// The wall snap: a packet moving toward the wall ahead whose coordinate is
// within 2 % of it (relative to the signed wall coordinate, as in the
// reference) is given the next cell index.
template <typename R>
__device__ __forceinline__ int axisSnap(const AxisVals<R>& A, int n, int a, R r, R v) {
  using M = RMath<R>;
  const R mUp = (A.c0 + A.p1) / R(2);
  const R mDn = (A.c0 + A.m1) / R(2);
  const bool up = a < n && v > R(0) && M::div_(M::abs_(r - mUp), mUp) < R(2.e-2);
  const bool dn = a > 1 && v < R(0) && M::div_(M::abs_(r - mDn), mDn) < R(2.e-2);
  return up ? a + 1 : (dn ? a - 1 : a);
}

template <typename R>
struct AxisStep { R r, v, dS; int a; bool lost; };

// The reflection at the first plane of a symmetric grid, then the distance to
// the wall ahead; a distance below 1e-5 puts the packet on that wall and in
// the next cell (lost beyond the grid's last plane).  a0 is the index the step
// started from (AxisVals holds the axis around it), a the index after the snap.
template <typename R>
__device__ __forceinline__ AxisStep<R> axisDistance(const AxisVals<R>& A, int n, int a0, int a, R r, R v,
                                                    bool symmetric, bool plane) {
  using M = RMath<R>;
  const bool refl = symmetric && r <= A.first;
  v = (refl && v < R(0)) ? -v : v;
  r = refl ? A.first : r;
  const int d = a - a0;                                        // -1, 0 or 1
  const R ca = d < 0 ? A.m1 : (d > 0 ? A.p1 : A.c0);           // A(a)
  const R cp = d < 0 ? A.c0 : (d > 0 ? A.p2 : A.p1);           // A(a+1)
  const R cm = d < 0 ? A.m2 : (d > 0 ? A.c0 : A.m1);           // A(a-1)
  const R wUp = (cp + ca) / R(2);
  const R wDn = (ca + cm) / R(2);
  const bool pos = v > R(0), neg = v < R(0);
  const R target = pos ? (a < n ? wUp : A.last) : (a > 1 ? wDn : A.first);
  const R dS = (pos || neg) ? M::div_(target - r, v) : A.last;
  const bool snap = (pos || neg) && M::abs_(dS) < R(1.e-5);
  AxisStep<R> o;
  o.r = snap ? target : r;
  o.v = v;
  o.dS = dS;
  o.a = snap ? (pos ? (a < n ? a + 1 : a) : (a > 1 ? a - 1 : a)) : a;
  o.lost = snap && pos && a >= n && !plane;   // a plane-parallel slab keeps it (source/photon_mod.f90:2003)
  return o;
}

// One iteration of pathSegment's main loop (source/photon_mod.f90:1880-4036);
// ST_ESCAPE when the packet leaves the grid or R_out (tallied by stepPacket).
template <typename R, typename Geo, typename P>
__device__ __forceinline__ int stepCore(const DevGrid& g, const Geo& q, const DevTransportIn& in,
                                          const DevTransportOut& out, const TransportShared<R>& sh, P& p,
                                          R deltaER, double deltaE, LocalCounters& lc, PendingJ& pj) {
  using M = RMath<R>;
  const int nx = q.nx(), ny = q.ny(), nz = q.nz();
  const float* X = q.X(); const float* Y = q.Y(); const float* Z = q.Z();
#define AXR(A, i) ((R)(A)[(i) - 1])
  // safeLimit: 5000 steps per segment for a plane-parallel slab (source/photon_mod.f90:1873-1878)
  if (++p.nStep > (q.plane() ? kSafeLimitPlane : kSafeLimit)) {
    ++lc.trapped;
    if (p.nEmit >= kRecursionLimit) ++lc.trapped;
    return ST_IDLE;
  }
  int xP = p.xP, yP = p.yP, zP = p.zP;
  if (xP < 1 || xP > nx || yP < 1 || yP > ny || zP < 1 || zP > nz) { ++lc.errors; return ST_IDLE; }
  R rx = p.x, ry = p.y, rz = p.z, vx = p.vx, vy = p.vy, vz = p.vz;

  // wall snap (source/photon_mod.f90:1882-1919), one axis at a time without
  // branches so that the three axes' arithmetic interleaves
  const int x0 = xP, y0 = yP, z0 = zP;
  const AxisVals<R> AX = axisLoad<R>(X, nx, xP), AY = axisLoad<R>(Y, ny, yP), AZ = axisLoad<R>(Z, nz, zP);
  xP = axisSnap<R>(AX, nx, xP, rx, vx);
  yP = axisSnap<R>(AY, ny, yP, ry, vy);
  zP = axisSnap<R>(AZ, nz, zP, rz, vz);

  // the opacity and volume of the cell the snap leaves the packet in, loaded
  // here so that their latency overlaps the wall-distance arithmetic; loaded
  // again below in the rare case that a distance snap moves the index
  const size_t C1 = (size_t)g.nCells + 1;
  int cell = activeAt(q, xP, yP, zP);
  R kap = (R)__ldg(in.opacity + (size_t)cell + C1 * (size_t)(p.nuP - 1));
  R dV = cell > 0 ? cellVolume<R>(g, cell) : R(1);
  const int xS = xP, yS = yP, zS = zP;
  // the scattering inputs: for a warp history loaded here with the opacity
  // (registers are plentiful there), for a trapped lane of the main kernel
  // prefetched into L1
  R scaIn = R(0), knIn = R(0), neIn = R(0);
  if constexpr (P::kWarp) {
    if (g.lgDust) scaIn = (R)__ldg(in.scaOpac + (size_t)cell + C1 * (size_t)(p.nuP - 1));
    else if (g.lgCompton) { knIn = (R)__ldg(g.KNsigmaT + p.nuP - 1); neIn = (R)__ldg(in.ne + cell); }
  } else if (p.nEmit > kTrappedHint) {
    if (g.lgDust) prefetchL1(in.scaOpac + (size_t)cell + C1 * (size_t)(p.nuP - 1));
    else if (g.lgCompton) { prefetchL1(g.KNsigmaT + p.nuP - 1); prefetchL1(in.ne + cell); }
  }

  // the symmetric grid's reflection and the distances from the walls
  // (source/photon_mod.f90:1921-2084); with one mother grid the reference's
  // inner loop runs exactly once
  const bool sym = q.symmetric() != 0, plane = q.plane();
  const AxisStep<R> sx = axisDistance<R>(AX, nx, x0, xP, rx, vx, sym, plane);
  const AxisStep<R> sy = axisDistance<R>(AY, ny, y0, yP, ry, vy, sym, plane);
  const AxisStep<R> sz = axisDistance<R>(AZ, nz, z0, zP, rz, vz, sym, plane);
  if (sx.lost || sy.lost || sz.lost) { if (p.nEmit >= kRecursionLimit) ++lc.trapped; return ST_IDLE; }
  rx = sx.r; vx = sx.v; xP = sx.a;
  ry = sy.r; vy = sy.v; yP = sy.a;
  rz = sz.r; vz = sz.v; zP = sz.a;
  R dSx = sx.dS, dSy = sy.dS, dSz = sz.dS;
  if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) { ++lc.errors; return ST_IDLE; }

  // nearest wall (source/photon_mod.f90:2087-2137)
  if (M::abs_(dSx) < R(1.e-5)) dSx = AXR(X, nx);
  if (M::abs_(dSy) < R(1.e-5)) dSy = AXR(Y, ny);
  if (M::abs_(dSz) < R(1.e-5)) dSz = AXR(Z, nz);
  dSx = M::abs_(dSx); dSy = M::abs_(dSy); dSz = M::abs_(dSz);
  R dS;
  if (dSx <= R(0)) dS = M::min_(dSy, dSz);
  else if (dSy <= R(0)) dS = M::min_(dSx, dSz);
  else if (dSz <= R(0)) dS = M::min_(dSx, dSy);
  else { dS = M::min_(dSx, dSy); dS = M::min_(dS, dSz); }
  if (!(dS > R(0))) { ++lc.errors; return ST_IDLE; }

  if (xP != xS || yP != yS || zP != zS) {
    cell = activeAt(q, xP, yP, zP);
    kap = (R)__ldg(in.opacity + (size_t)cell + C1 * (size_t)(p.nuP - 1));
    dV = cell > 0 ? cellVolume<R>(g, cell) : R(1);
    if constexpr (P::kWarp) {
      if (g.lgDust) scaIn = (R)__ldg(in.scaOpac + (size_t)cell + C1 * (size_t)(p.nuP - 1));
      else if (g.lgCompton) neIn = (R)__ldg(in.ne + cell);
    }
  }
  const R tauCell = dS * kap;
  R costheta = R(1);
  if (g.radPress && !(rx == R(0) && ry == R(0) && rz == R(0))) {
    costheta = ((rx * vx) + (ry * vy) + (rz * vz)) /
               (R(1.e10) * M::sqrt_((rx / R(1.e10)) * (rx / R(1.e10)) + (ry / R(1.e10)) * (ry / R(1.e10)) +
                                    (rz / R(1.e10)) * (rz / R(1.e10))));
  }

  int next = ST_STEP;
  if ((p.absTau + tauCell > p.passProb) && cell > 0) {
    // interaction within the cell (source/photon_mod.f90:2244-2700)
    R dlLoc = M::div_(p.passProb - p.absTau, kap);
    rx = rx + dlLoc * vx; ry = ry + dlLoc * vy; rz = rz + dlLoc * vz;
    if (q.symmetric()) {
      if (rx <= AXR(X, 1)) { if (vx < R(0)) vx = -vx; rx = AXR(X, 1); }
      if (ry <= AXR(Y, 1)) { if (vy < R(0)) vy = -vy; ry = AXR(Y, 1); }
      if (rz <= AXR(Z, 1)) { if (vz < R(0)) vz = -vz; rz = AXR(Z, 1); }
    }
    deposit<R, P::kWarp>(g, out, cell, p.nuP, dlLoc, dV, deltaER, costheta, pj);
    ++lc.interactions;
    // the radius only matters against an outer radius R_out > 0
    if (q.rOut() > 0.f &&
        M::sqrt_((rx / R(1.e10)) * (rx / R(1.e10)) + (ry / R(1.e10)) * (ry / R(1.e10)) +
                 (rz / R(1.e10)) * (rz / R(1.e10))) * R(1.e10) >= (R)q.rOut()) {
      return ST_ESCAPE;
    }
    if (g.lgDust) {
      R probSca = (P::kWarp ? scaIn : (R)__ldg(in.scaOpac + (size_t)cell + C1 * (size_t)(p.nuP - 1))) / kap;
      R rnd = R(1) - draw(p);
      if (rnd > probSca) {
        ++lc.absorptions;
        p.type = g.lgGas ? PT_DIFFUSE : PT_DUSTEMI;
        next = ST_EMIT;
      } else {
        ++lc.scatterings;
        initPacket<R>(q, sh, p, p.nuP, false, false, xP, yP, zP);
        vx = p.vx; vy = p.vy; vz = p.vz;
        p.absTau = R(0);
        p.passProb = drawPassProb(p);
      }
    } else {
      R probSca = R(0);
      if (g.lgCompton) {
        if constexpr (P::kWarp) probSca = knIn * neIn / kap;
        else probSca = (R)__ldg(g.KNsigmaT + p.nuP - 1) * (R)__ldg(in.ne + cell) / kap;
      }
      R rnd = R(1) - draw(p);
      if (rnd <= probSca) {
        ++lc.scatterings;
        comptonScatter<R>(g, sh, p);
        p.origin = cell;
        vx = p.vx; vy = p.vy; vz = p.vz;
        p.absTau = R(0);
        p.passProb = drawPassProb(p);
      } else {
        ++lc.absorptions;
        p.type = PT_DIFFUSE;
        next = ST_EMIT;
      }
    }
  } else {
    // the packet crosses the cell (source/photon_mod.f90:2703-2881)
    deposit<R, P::kWarp>(g, out, cell, p.nuP, dS, dV, deltaER, costheta, pj);
    ++lc.crossings;
    p.absTau = p.absTau + tauCell;
    rx = rx + dS * vx; ry = ry + dS * vy; rz = rz + dS * vz;
    if (dS == dSx && vx > R(0)) xP = xP + 1;
    else if (dS == dSx && vx < R(0)) xP = xP - 1;
    else if (dS == dSy && vy > R(0)) yP = yP + 1;
    else if (dS == dSy && vy < R(0)) yP = yP - 1;
    else if (dS == dSz && vz > R(0)) zP = zP + 1;
    else if (dS == dSz && vz < R(0)) zP = zP - 1;
    bool esc = false;
    if (q.plane()) {
      // plane-parallel slab (source/photon_mod.f90:3249-3611): out through the
      // y planes only, reflected at the x and z planes (the lower z plane puts
      // z at yAxis(1), as the reference does)
      if (ry < AXR(Y, 1) || yP < 1) { yP = 1; esc = true; }
      if (ry > AXR(Y, ny) || yP > ny) { yP = ny; esc = true; }
      if (rx <= AXR(X, 1) || xP < 1) { xP = 1; rx = AXR(X, 1); vx = -vx; }
      if (rx >= AXR(X, nx) || xP > nx) { xP = nx; rx = AXR(X, nx); vx = -vx; }
      if (rz <= AXR(Z, 1) || zP < 1) { zP = 1; rz = AXR(Y, 1); vz = -vz; }
      if (rz >= AXR(Z, nz) || zP > nz) { zP = nz; rz = AXR(Z, nz); vz = -vz; }
      if (esc) return ST_ESCAPE;
    } else {
      if (!q.symmetric()) {
        // full-grid escape (source/photon_mod.f90:2884-3244)
        if (ry < AXR(Y, 1) || yP < 1) esc = true;
        if (ry > AXR(Y, ny) || yP > ny) esc = true;
        if (rx <= AXR(X, 1) || xP < 1) esc = true;
        if (rx >= AXR(X, nx) || xP > nx) esc = true;
        if (rz <= AXR(Z, 1) || zP < 1) esc = true;
        if (rz >= AXR(Z, nz) || zP > nz) esc = true;
      }
      // grid boundary and mirror planes (source/photon_mod.f90:3607-3890)
      if (!esc && ((!q.symmetric() && (rx <= AXR(X, 1) || ry <= AXR(Y, 1) || rz <= AXR(Z, 1))) ||
                   rx >= AXR(X, nx) || ry >= AXR(Y, ny) || rz >= AXR(Z, nz) || xP > nx || yP > ny || zP > nz))
        esc = true;
      if (esc) return ST_ESCAPE;
      if (q.symmetric()) {
        if (rx <= AXR(X, 1) || xP < 1) { if (vx < R(0)) vx = -vx; xP = 1; rx = AXR(X, 1); }
        if (ry <= AXR(Y, 1) || yP < 1) { if (vy < R(0)) vy = -vy; yP = 1; ry = AXR(Y, 1); }
        if (rz <= AXR(Z, 1) || zP < 1) { if (vz < R(0)) vz = -vz; zP = 1; rz = AXR(Z, 1); }
      }
    }
  }
  // source/photon_mod.f90:3951-4036
  if (next == ST_STEP && !q.plane() && (xP > nx || yP > ny || zP > nz)) {
    return ST_ESCAPE;
  }
  p.x = rx; p.y = ry; p.z = rz; p.vx = vx; p.vy = vy; p.vz = vz;
  p.xP = xP; p.yP = yP; p.zP = zP;
  return next;
#undef AXR
}

// A step and, for a packet that leaves, its escape tally (one copy of it).
template <typename R, typename Geo, typename P>
__device__ __forceinline__ int stepPacket(const DevGrid& g, const Geo& q, const DevTransportIn& in,
                                          const DevTransportOut& out, const TransportShared<R>& sh, P& p,
                                          R deltaER, double deltaE, LocalCounters& lc, PendingJ& pj) {
  const int st = stepCore<R>(g, q, in, out, sh, p, deltaER, deltaE, lc, pj);
  if (st != ST_ESCAPE) return st;
  escapeTally<R>(g, out, p, deltaE, lc);
  if (p.nEmit >= kRecursionLimit) ++lc.trapped;
  return ST_IDLE;
}

// one atomic per counter per warp
__device__ __forceinline__ void flushCounters(const LocalCounters& lc, DevTransportCounters* cnt) {
  const unsigned FULL = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  auto wsum = [&](unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    return v;
  };
  unsigned long long v;
  v = wsum(lc.crossings);    if (lane == 0 && v) atomicAdd(&cnt->crossings, v);
  v = wsum(lc.interactions); if (lane == 0 && v) atomicAdd(&cnt->interactions, v);
  v = wsum(lc.absorptions);  if (lane == 0 && v) atomicAdd(&cnt->absorptions, v);
  v = wsum(lc.scatterings);  if (lane == 0 && v) atomicAdd(&cnt->scatterings, v);
  v = wsum(lc.escaped);      if (lane == 0 && v) atomicAdd(&cnt->escaped, v);
  v = wsum(lc.lineEscapes);  if (lane == 0 && v) atomicAdd(&cnt->lineEscapes, v);
  v = wsum(lc.trapped);      if (lane == 0 && v) atomicAdd(&cnt->trapped, v);
  v = wsum(lc.emissions);    if (lane == 0 && v) atomicAdd(&cnt->emissions, v);
  v = wsum(lc.errors);       if (lane == 0 && v) atomicAdd(&cnt->errors, v);
  double qp = lc.qPhot;
  for (int o = 16; o > 0; o >>= 1) qp += __shfl_down_sync(FULL, qp, o);
  if (lane == 0 && qp != 0.) atomicAdd(&cnt->qPhot, qp);
}

// Emission and cell steps take turns by warp: an iteration runs the emission
// code only once kEmitBatch lanes wait for it (or no lane is stepping), else
// it runs one cell step of every stepping lane.  Emissions are about one event
// in ten but long (a CDF bisection through global memory, the direction
// draw); run one lane at a time they would stall the other 31 lanes on almost
// every iteration.  Only the order of events across lanes changes, not any
// packet's history.
constexpr int kEmitBatch = 12;   // default; the launch may choose another

__device__ __forceinline__ bool emitTurn(int state, int emitBatch) {
  const unsigned FULL = 0xffffffffu;
  const unsigned emit = __ballot_sync(FULL, state == ST_EMIT);
  const unsigned step = __ballot_sync(FULL, state == ST_STEP);
  return emit != 0u && (__popc(emit) >= emitBatch || step == 0u);
}

// Idle lanes of the warp take the next packet ids from the work queue with one
// atomic; returns this lane's id (meaningful when the lane was idle).
__device__ __forceinline__ unsigned long long refill(unsigned need, DevTransportCounters* cnt) {
  const unsigned FULL = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  const int leader = __ffs(need) - 1;
  unsigned long long first = 0;
  if ((int)lane == leader) first = atomicAdd(&cnt->queue, (unsigned long long)__popc(need));
  first = __shfl_sync(FULL, first, leader);
  return first + (unsigned long long)__popc(need & ((1u << lane) - 1u));
}

template <typename R, bool kPlane>
__global__ void __launch_bounds__(256)
transportKernel(DevGrid g, DevTransportIn in, DevTransportOut out, DevTransportCounters* cnt,
                uint64_t seed, uint64_t base, unsigned long long n, double deltaE, int emitBatch,
                Packet<R>* __restrict__ parked, unsigned long long parkedCap, int handoffAt) {
  extern __shared__ float smem[];
  float* sX = smem;
  float* sY = sX + g.nx;
  float* sZ = sY + g.ny;
  float* sNu = sZ + g.nz;
  float* sCdf = sNu + g.nbins;
  for (int i = threadIdx.x; i < g.nx; i += blockDim.x) sX[i] = g.xAxis[i];
  for (int i = threadIdx.x; i < g.ny; i += blockDim.x) sY[i] = g.yAxis[i];
  for (int i = threadIdx.x; i < g.nz; i += blockDim.x) sZ[i] = g.zAxis[i];
  for (int i = threadIdx.x; i < g.nbins; i += blockDim.x) { sNu[i] = g.nu[i]; sCdf[i] = g.srcCDF[i]; }
  __syncthreads();
  TransportShared<R> sh{sNu};
  const OneGrid<kPlane> q{g, sX, sY, sZ, sCdf};

  const unsigned FULL = 0xffffffffu;
  const R deltaER = (R)deltaE;
  LocalCounters lc;
  Packet<R>& p = reinterpret_cast<Packet<R>*>(
      reinterpret_cast<char*>(smem) +
      packetStateOffset((size_t)(g.nx + g.ny + g.nz + 2 * g.nbins) * sizeof(float)))[threadIdx.x];
  p.nEmit = 0; p.nStep = 0;
  PendingJ pj{0., 0., 0, false};
  int state = ST_IDLE;

  for (;;) {
    const unsigned need = __ballot_sync(FULL, state == ST_IDLE);
    if (need) {
      const unsigned long long id = refill(need, cnt);
      if (state == ST_IDLE) {
        if (id < n) {
          p.rng.init(seed, base + id);
          p.type = PT_STELLAR;
          p.nEmit = 0;
          state = ST_EMIT;
        } else {
          state = ST_DONE;
        }
      }
    }
    if (__ballot_sync(FULL, state != ST_DONE) == 0u) break;
    if (emitTurn(state, emitBatch)) {
      if (state == ST_EMIT) {
        bool moved = false;
        if (handoffAt > 0 && p.nEmit >= handoffAt && p.nEmit < kRecursionLimit) {
          // trapped: park the history here, as it stands before this emission,
          // for the trapped-packet kernel, and take the next packet
          const unsigned long long slot = atomicAdd(&cnt->handoff, 1ull);
          if (slot < parkedCap) { parked[slot] = p; state = ST_IDLE; moved = true; }
        }
        if (!moved) state = emitPacket<R>(g, q, in, out, sh, p, deltaE, lc);
      }
    } else if (state == ST_STEP) {
      state = stepPacket<R>(g, q, in, out, sh, p, deltaER, deltaE, lc, pj);
    }
  }
  flushJ(out, pj);
  flushCounters(lc, cnt);
}

// The trapped-packet kernel, launched after transportKernel on the same stream:
// continues every parked history to its end, one history per warp (one warp
// per block, as many blocks as are resident at once, histories handed out
// round-robin).  A trapped history is a serial chain of up to recursionLimit
// emission + step events whose length sets the launch's; a lone lane runs that
// chain at one instruction per several cycles, so the warp's other lanes are
// put to work on its data-parallel parts (the Philox stream, the CDF search)
// while all lanes run the scalar physics in lockstep.  No shared memory: axes
// and frequencies are read through L1, which keeps its full size.
template <typename R, bool kPlane>
__global__ void __launch_bounds__(32, 16)   // 16 histories per SM, 2432 at once on 152 SMs: no spills at 128 registers
transportTrappedKernel(DevGrid g, DevTransportIn in, DevTransportOut out, DevTransportCounters* cnt, double deltaE,
                       const Packet<R>* __restrict__ parked, unsigned long long parkedCap,
                       unsigned long long warpMax) {
  const unsigned long long written = *reinterpret_cast<volatile unsigned long long*>(&cnt->handoff);
  const unsigned long long count = written < parkedCap ? written : parkedCap;
  // many more histories than resident warps: transportTrappedLanesKernel runs them
  if (count > warpMax) return;
  TransportShared<R> sh{g.nu};
  const OneGrid<kPlane> q{g, g.xAxis, g.yAxis, g.zAxis, g.srcCDF};
  const R deltaER = (R)deltaE;
  LocalCounters lc;
  PendingJ pj{0., 0., 0, false};
  // the first gridDim.x histories one per warp, the rest from a queue as
  // warps finish (most parked histories end within a few hundred events; a
  // trapped one runs to recursionLimit)
  const int2 cdfShape = warpCdfShape(g.nbins);
  for (unsigned long long i = blockIdx.x; i < count;) {
    WarpPacket<R> p;
    p.from(parked[i]);
    p.cdfShape = cdfShape;
    int state = ST_EMIT;
    while (state == ST_EMIT || state == ST_STEP) {
      if (state == ST_EMIT) state = emitBody<R, OneGrid<kPlane>>(g, q, in, out, sh, p, deltaE, lc);
      else state = stepPacket<R>(g, q, in, out, sh, p, deltaER, deltaE, lc, pj);
    }
    unsigned long long nxt = 0;
    if ((threadIdx.x & 31u) == 0u) nxt = gridDim.x + atomicAdd(&cnt->parkedNext, 1ull);
    i = __shfl_sync(0xffffffffu, nxt, 0);
  }
  flushJ(out, pj);
  if ((threadIdx.x & 31u) != 0u) lc = LocalCounters{};   // every lane counted the same events
  flushCounters(lc, cnt);
}

// The trapped-packet kernel for many parked histories (more than the warp
// kernel holds resident at once, e.g. tens of thousands on an X-ray-heated
// grid): one history per lane, taken from the parked queue as lanes free up,
// with the main kernel's emission batching; the warp kernel's single-history
// latency matters less here than running every history at once.  Histories
// in registers, event code inlined, no shared memory.
template <typename R, bool kPlane>
__global__ void __launch_bounds__(128)
transportTrappedLanesKernel(DevGrid g, DevTransportIn in, DevTransportOut out, DevTransportCounters* cnt,
                            double deltaE, const Packet<R>* __restrict__ parked, unsigned long long parkedCap,
                            unsigned long long warpMax, int emitBatch) {
  const unsigned long long written = *reinterpret_cast<volatile unsigned long long*>(&cnt->handoff);
  const unsigned long long count = written < parkedCap ? written : parkedCap;
  if (count <= warpMax) return;   // transportTrappedKernel has them, one per warp
  TransportShared<R> sh{g.nu};
  const OneGrid<kPlane> q{g, g.xAxis, g.yAxis, g.zAxis, g.srcCDF};
  const R deltaER = (R)deltaE;
  const unsigned FULL = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  LocalCounters lc;
  PendingJ pj{0., 0., 0, false};
  Packet<R> p;
  p.nEmit = 0;
  int state = ST_IDLE;
  for (;;) {
    const unsigned need = __ballot_sync(FULL, state == ST_IDLE);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long first = 0;
      if ((int)lane == leader) first = atomicAdd(&cnt->parkedNext, (unsigned long long)__popc(need));
      first = __shfl_sync(FULL, first, leader);
      const unsigned long long id = first + (unsigned long long)__popc(need & ((1u << lane) - 1u));
      if (state == ST_IDLE) {
        if (id < count) { p = parked[id]; state = ST_EMIT; }
        else state = ST_DONE;
      }
    }
    if (__ballot_sync(FULL, state != ST_DONE) == 0u) break;
    if (emitTurn(state, emitBatch)) {
      if (state == ST_EMIT) state = emitBody<R, OneGrid<kPlane>>(g, q, in, out, sh, p, deltaE, lc);
    } else if (state == ST_STEP) {
      state = stepPacket<R>(g, q, in, out, sh, p, deltaER, deltaE, lc, pj);
    }
  }
  flushJ(out, pj);
  flushCounters(lc, cnt);
}

// A batch of nebulae sharing one frequency mesh and chemistry: their cells are
// numbered batch-wide (the per-cell arrays are the concatenation of the
// nebulae's), and packet ids are handed out batch-wide, nebula b owning
// [pktBegin[b], pktBegin[b+1]).  A lane that takes a packet looks up its
// nebula (bisection over the batch), then runs the same emit / step code in
// that nebula's geometry with its own deltaE = L*/nPhotons and its own Philox
// key and counter base, so every nebula's histories are those of a run of the
// nebula alone.
__device__ __forceinline__ unsigned long long globalTimerNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The GPU's global timer when the batched launch begins (one thread, launched
// on the same stream just before it).
static __global__ void stampStartKernel(unsigned long long* startNs) { *startNs = globalTimerNs(); }

template <typename R>
__global__ void __launch_bounds__(256, 4)
transportKernelBatched(DevGrid g, DevTransportIn in, DevTransportOut out, DevTransportCounters* cnt,
                       const NebulaDesc* __restrict__ neb, const unsigned long long* __restrict__ pktBegin, int nNeb,
                       const float* __restrict__ axes, const int32_t* __restrict__ active,
                       const float* __restrict__ cdfs, int emitBatch, unsigned long long* __restrict__ doneNs) {
  extern __shared__ float smem[];
  float* sNu = smem;
  for (int i = threadIdx.x; i < g.nbins; i += blockDim.x) sNu[i] = g.nu[i];
  __syncthreads();
  TransportShared<R> sh{sNu};
  const unsigned long long n = pktBegin[nNeb];

  const unsigned FULL = 0xffffffffu;
  LocalCounters lc;
  Packet<R>& p = reinterpret_cast<Packet<R>*>(reinterpret_cast<char*>(smem) +
                                              packetStateOffset((size_t)g.nbins * sizeof(float)))[threadIdx.x];
  p.nEmit = 0; p.nStep = 0;
  NebulaGeo q{};
  PendingJ pj{0., 0., 0, false};
  double deltaE = 0.;
  R deltaER = R(0);
  int state = ST_IDLE;
  int mine = -1;              // the nebula of the lane's packet in flight
  // the latest finish among this lane's packets of nebula stampNeb, published
  // with one atomic when the lane moves on to another nebula (packet ids, and
  // so the nebulae, are handed out in order) or leaves
  int stampNeb = -1;
  unsigned long long stampNs = 0ull;

  for (;;) {
    if (state == ST_IDLE && mine >= 0) {
      if (mine != stampNeb) {
        if (stampNeb >= 0) atomicMax(doneNs + stampNeb, stampNs);
        stampNeb = mine;
      }
      stampNs = globalTimerNs();
      mine = -1;
    }
    const unsigned need = __ballot_sync(FULL, state == ST_IDLE);
    if (need) {
      const unsigned long long id = refill(need, cnt);
      if (state == ST_IDLE) {
        if (id < n) {
          int lo = 0, hi = nNeb - 1;      // last b with pktBegin[b] <= id
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(pktBegin + mid) <= id) lo = mid; else hi = mid - 1;
          }
          const NebulaDesc& d = neb[lo];
          q.nx_ = d.nx; q.ny_ = d.ny; q.nz_ = d.nz; q.symmetric_ = d.symmetric; q.rOut_ = d.rOut;
          q.X_ = axes + d.axOff; q.Y_ = q.X_ + d.nx; q.Z_ = q.Y_ + d.ny;
          q.active_ = active + d.actOff;
          q.cdf_ = cdfs + d.cdfOff;
          for (int k = 0; k < 3; ++k) { q.starIdx_[k] = d.starIdx[k]; q.starPos_[k] = d.starPos[k]; }
          deltaE = d.deltaE;
          deltaER = (R)deltaE;
          p.rng.init(d.seed, d.counterBase + (id - __ldg(pktBegin + lo)));
          mine = lo;
          p.type = PT_STELLAR;
          p.nEmit = 0;
          state = ST_EMIT;
        } else {
          state = ST_DONE;
        }
      }
    }
    if (__ballot_sync(FULL, state != ST_DONE) == 0u) break;
    if (emitTurn(state, emitBatch)) {
      if (state == ST_EMIT) state = emitPacket<R>(g, q, in, out, sh, p, deltaE, lc);
    } else if (state == ST_STEP) {
      state = stepPacket<R>(g, q, in, out, sh, p, deltaER, deltaE, lc, pj);
    }
  }
  if (stampNeb >= 0) atomicMax(doneNs + stampNeb, stampNs);
  flushJ(out, pj);
  flushCounters(lc, cnt);
}

// The single-grid launch: the persistent kernel, then, when hand-off is on,
// the trapped-packet kernel with one warp per block on every SM (as many
// blocks as are resident at once, so every parked history starts at once).
template <typename R, bool kPlane>
cudaError_t launchTransportPlane(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                                double deltaE, const TransportLaunch& L, cudaStream_t s) {
  const size_t smem = packetStateOffset(L.smem) + packetStateBytes<R>(L.threads);
  cudaError_t e = cudaFuncSetAttribute(transportKernel<R, kPlane>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const bool hand = L.parked != nullptr && L.parkedCap > 0 && L.handoffAt > 0 && L.numSMs > 0;
  transportKernel<R, kPlane><<<L.blocks, L.threads, smem, s>>>(g, in, out, cnt, seed, base, n, deltaE,
                                                       L.emitBatch > 0 ? L.emitBatch : kEmitBatch,
                                                       hand ? static_cast<Packet<R>*>(L.parked) : nullptr,
                                                       hand ? L.parkedCap : 0ull, hand ? L.handoffAt : 0);
  e = cudaGetLastError();
  if (e != cudaSuccess || !hand) return e;
  // both continuation kernels; each reads the parked count and only one works:
  // one history per warp up to three times the resident warps (most parked
  // histories end within a few hundred events, so the queue keeps the
  // trapped ones running in the first waves; measured on the 41^3 lognormal
  // run), one per lane beyond (the 41^3 X-ray run parks ~2e4 trapped histories,
  // which would take ten waves one per warp)
  int perSM = 0, lanesPerSM = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, transportTrappedKernel<R, kPlane>, 32, 0);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lanesPerSM, transportTrappedLanesKernel<R, kPlane>, 128, 0);
  if (e != cudaSuccess) return e;
  if (perSM < 1) perSM = 1;
  if (lanesPerSM < 1) lanesPerSM = 1;
  const unsigned long long warpSlots = (unsigned long long)L.numSMs * perSM;
  const unsigned long long warpMax = 3 * warpSlots;
  transportTrappedKernel<R, kPlane><<<(unsigned)warpSlots, 32, 0, s>>>(g, in, out, cnt, deltaE,
                                                               static_cast<const Packet<R>*>(L.parked), L.parkedCap,
                                                               warpMax);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  transportTrappedLanesKernel<R, kPlane><<<L.numSMs * lanesPerSM, 128, 0, s>>>(
      g, in, out, cnt, deltaE, static_cast<const Packet<R>*>(L.parked), L.parkedCap, warpMax,
      L.emitBatch > 0 ? L.emitBatch : kEmitBatch);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launchTransportImpl(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                                double deltaE, const TransportLaunch& L, cudaStream_t s) {
  return g.plane ? launchTransportPlane<R, true>(g, in, out, cnt, seed, base, n, deltaE, L, s)
                 : launchTransportPlane<R, false>(g, in, out, cnt, seed, base, n, deltaE, L, s);
}

}  // namespace mcx
