// tsph_internal.cuh -- device-side types and helpers shared by the kernels.
//
// Data layout in HBM (one system):
//   fluid  : structure-of-arrays sorted by cell id (counting sort, stable by
//            particle index).  r is FP64 (double2); v, a, rho, drho, p are T
//            (float in the production build, double in the FP64 build).  In
//            the float build `rho` holds rho - rho0, which keeps ~5 more bits
//            of the density than a float rho would (rho ~ 1000, changes ~1e-3).
//            loc = position relative to the particle's cell origin in FP32,
//            so the pair kernels form r_a - r_b without FP64 arithmetic
//            (GB300 runs FP64 at 1/64 of the FP32 rate).
//   walls  : the same fields, binned once (walls never move), plus the mDBC
//            ghost node and its cell.
//   cells  : fstart[ncells+2] (fluid CSR offsets, last bucket = removed
//            particles), wstart[ncells+1] (walls).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

namespace tsph {

constexpr int kBlock = 256;

template <typename T> struct V2;
template <> struct V2<float> { typedef float2 t; };
template <> struct V2<double> { typedef double2 t; };

// ------------------------------------------------------------------ grid
// Cell id of a coordinate, exactly as the reference computes it
// ((int)((x - x_0 + of)/kh), src/SPH_find_pairs.h:64-65) but without FP64
// division: that expression is a monotone step function of the double x, so
// the host tabulates, per axis, the smallest double at which each cell index
// begins (bisection over the ordered doubles, evaluating the very same FP64
// expression), and the device compares the bits of x against the table.
struct Axis {
    const long long *bnd;  // n+1 ordered-int64 lower bounds: cell k = [bnd[k], bnd[k+1])
    const double *org;     // n cell origins x_0 - of + k*kh (FP64)
    int n;
};

struct Grid {
    Axis ax, ay;
    int ncx, ncy, ncells;
    float khf;  // kh rounded to float (cell-to-cell offset in the pair kernels)
};

// monotone map of a double's bits to a signed 64-bit integer
__host__ __device__ inline long long ordered_bits(double x) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(x);
#else
    long long b;
    memcpy(&b, &x, 8);
#endif
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// Programmatic dependent launch.  Every kernel the engine launches starts
// here: it waits until the previous kernel of the stream has completed and
// its writes are visible (a no-op when it was launched without the
// programmatic-serialisation attribute), then lets the next kernel of the
// stream begin launching, so that kernel's launch and block scheduling
// overlap this one's tail instead of following it.  Nothing is read or
// written before the wait.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ inline bool is_finite_d(double x) {
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

// index of the cell along one axis, or -1 below / n above the grid.
// `guess` is any starting index (e.g. the previous cell); the walk is bounded.
__device__ inline int axis_cell(const Axis &a, double x, int guess) {
    const long long o = ordered_bits(x);
    if (o < __ldg(a.bnd)) return -1;
    if (o >= __ldg(a.bnd + a.n)) return a.n;
    int k = min(max(guess, 0), a.n - 1);
    // at most a few steps when the guess is the previous cell
    if (o < __ldg(a.bnd + k)) {
        int lo = 0, hi = k;  // answer in [lo, hi)
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (o < __ldg(a.bnd + mid)) hi = mid; else lo = mid;
        }
        return lo;
    }
    if (o >= __ldg(a.bnd + k + 1)) {
        int lo = k + 1, hi = a.n;  // answer in [lo, hi)
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (o < __ldg(a.bnd + mid)) hi = mid; else lo = mid;
        }
        return lo;
    }
    return k;
}

// ------------------------------------------------------------------ state
template <typename T> struct FluidState {
    double2 *r;
    typename V2<T>::t *v, *a;
    T *rho, *drho, *p;
    uint32_t *id;   // original particle index
    uint32_t *key;  // cell id (ncells = removed)
    float2 *loc;    // r - cell origin, FP32
    uint8_t *type = nullptr;  // particle type (systems with buffer zones only; 0 = fluid)
};

template <typename T> struct OldState {  // r_o, v_o, rho_o of the predictor
    double2 *r;
    typename V2<T>::t *v;
    T *rho;
};

template <typename T> struct WallState {
    double2 *r;
    float2 *loc;
    uint32_t *key, *id;
    T *rho, *drho, *p, *rho_o;
    double2 *gnr;    // ghost node
    uint32_t *gkey;  // ghost node cell (ncells if outside the grid)
    float2 *gloc;    // ghost node - its cell origin
    typename V2<T>::t *gnd;  // r - gnr
};

// the (padded) domain box of Simulation_data
struct Box {
    double x0, xm, y0, ym;
};

// the thresholds of RemoveParticlesOutOfDomain (x0 - eps, xm - eps, y0 - eps,
// ym + eps with eps = 0.01, src/SPH_btdebug.h:16-19) as ordered bits
struct BoxBits {
    long long x_lo, x_hi, y_lo, y_hi;
};

// physical constants in both precisions
template <typename T> struct Phys {
    double hd;             // h in FP64 (exact pair-set tests)
    T h, inv_h, kh, m, c0, alpha, delta, rho0, g;
    T awen, bwen;          // Wendland constants rounded through float (src/SPH_kernel.h:56-57)
    T four_h2, eps_h2;     // (2h)^2, eps*h^2 (eps = 0.01, src/SPH_defs.h:69)
    T bwen_h;              // bwen / h: (dW/dr)/r = bwen (1-q/2)^3 / h
    T b_eos;               // c0^2 rho0 / 7
    T k_av;                // -2 alpha c0 h        (AV with mean density 0.5(ra+rb))
    T k_psi;               // 2 c0 h delta         (Fourtakas psi prefactor)
    T xg;                  // rho0 g / cb = 7 g / c0^2 (hydrostatic term argument per metre)
    T dp;                  // particle spacing (boundary-integral wall terms)
};

// density as stored -> full density
template <typename T> __device__ __forceinline__ T rho_full(T s, T rho0) {
    if constexpr (std::is_same<T, float>::value) return rho0 + s;
    else return s;
}
// the same in FP64 (what the host reads: rho0 + s rounded to float would
// drop the low bits of s, ~6e-5 kg/m^3 at rho ~ 1000)
template <typename T> __device__ __forceinline__ double rho_full64(T s, T rho0) {
    if constexpr (std::is_same<T, float>::value) return (double)rho0 + (double)s;
    else return s;
}
template <typename T> __host__ __device__ __forceinline__ T rho_stored_from_full(double full, double rho0) {
    if constexpr (std::is_same<T, float>::value) return (float)(full - rho0);
    else return full;
}

// Tait EOS, src/SPH_pressure.h:7-21.  Float build: B((1+s)^7 - 1) with
// s = (rho - rho0)/rho0 expanded by the binomial theorem (no cancellation).
template <typename T> __device__ __forceinline__ T eos(T stored, const Phys<T> &P) {
    if constexpr (std::is_same<T, float>::value) {
        const float s = stored / P.rho0;
        const float poly = s * (7.f + s * (21.f + s * (35.f + s * (35.f + s * (21.f + s * (7.f + s))))));
        return P.b_eos * poly;
    } else {
        const double gamma = 7.;
        const double b_const = P.c0 * P.c0 * P.rho0 / gamma;
        const double rho_r = stored / P.rho0;
        return b_const * (pow(rho_r, gamma) - 1);
    }
}

// device health word bits (mirror TSPH_HEALTH_* in tsph.h)
constexpr uint32_t kHealthNan = 0x1u, kHealthDensity = 0x2u, kHealthEscaped = 0x4u,
                   kHealthRemoved = 0x8u, kHealthStall = 0x10u,
                   kHealthUpload = 0x20u;

}  // namespace tsph
