// bs_noalloc.cu -- nonbonded forces and energies of a small system by direct summation over all
// pairs, with every byte of scratch memory in one fixed-size array of this module, so that a call
// allocates nothing.
//
// Who needs it. A handle (bs_create/bs_setup) owns growable device buffers: pair lists, cell
// arrays, energy partials. Some callers cannot let a library allocate behind their back:
//   * a host application that manages all device memory through its own pool (a caching
//     allocator, a visualisation or steering front-end) and must keep its budget exact;
//   * an interactive loop that evaluates forces inside a fixed frame budget, where a device
//     allocation may synchronise the whole device and stall the frame;
//   * code that runs when the device is nearly full, where an allocation can fail at a point the
//     caller cannot recover from.
// Such callers pass device buffers they own; this entry point only reads and writes those and
// its own static scratch.
//
// The terms follow the reference force loop for one dynamic particle i
// (src/spn/SpringNetwork.cpp:93-198, src/spn/Particle.cpp:191-253, 269-330, 368-429):
// every other particle j within the term's cutoff acts on i; a dynamic partner's pair energy is
// shared half and half, a static partner's is counted in full at i; static particles get no
// force. Pair kernels: src/forcefield/energy/steric.hpp:27-156,
// electrostatic.hpp:16-49 (plus the eps = D r extension), hydrophobic.hpp:20-39.
// There is no spring topology here, so no pair is excluded: the result is the one a handle
// with spring.enable = 0 gives.

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "bs_common.cuh"

namespace bsg
{
namespace
{

constexpr int kNaMaxN = BS_NOALLOC_MAX_PARTICLES;
constexpr int kNaBlock = 64;                         // threads per block, one particle each
constexpr int kNaMaxBlocks = kNaMaxN / kNaBlock;     // 256
constexpr int kNaTerms = 3;                          // steric, Coulomb, hydrophobic

// Scratch layout (byte offsets into na_scratch):
//   [kNaPosOff]  float4 [kNaMaxN]  x, y, z, steric factor P (the radius in linear mode)
//   [kNaPrmOff]  float4 [kNaMaxN]  steric factor F, charge, hydrophobicity, flag bits
//   [kNaBlkOff]  double [kNaMaxBlocks][kNaTerms]  per-block energy partials (overwritten)
//   [kNaDoneOff] unsigned int  blocks finished in the current call; must be 0 when a call
//                starts: set-up clears it, and the last block of every call puts it back to 0.
constexpr size_t kNaPosOff = 0;
constexpr size_t kNaPrmOff = kNaPosOff + sizeof(float4) * kNaMaxN;
constexpr size_t kNaBlkOff = kNaPrmOff + sizeof(float4) * kNaMaxN;
constexpr size_t kNaDoneOff = kNaBlkOff + sizeof(double) * kNaMaxBlocks * kNaTerms;
constexpr size_t kNaBytes = (kNaDoneOff + sizeof(unsigned int) + 255) / 256 * 256; // 518 KB

static __device__ __align__(256) unsigned char na_scratch[kNaBytes];

struct NaParams
{
    int n;
    int steric_on, coulomb_on, hydro_on;
    int steric_mode, dist_dielectric;
    float c_steric, c_coulomb, c_hydro;
    float lo2_s, hi2_s, lo2_c, hi2_c, lo2_h, hi2_h;
    float kf_steric, ke_steric;     // force and energy factors of each term
    float kf_elec, ke_elec;
    float kf_hydro, ke_hydro;
};

struct NaBuffers
{
    float4 *pos;
    float4 *prm;
    double *blk;
    unsigned int *done;
};

__host__ __device__ inline NaBuffers na_buffers(unsigned char *base)
{
    NaBuffers b;
    b.pos = reinterpret_cast<float4 *>(base + kNaPosOff);
    b.prm = reinterpret_cast<float4 *>(base + kNaPrmOff);
    b.blk = reinterpret_cast<double *>(base + kNaBlkOff);
    b.done = reinterpret_cast<unsigned int *>(base + kNaDoneOff);
    return b;
}

// The reference's pair test for one cutoff: FP64 distance of the float coordinates
// (nsearch.hpp:230), then the float-rounded FP64 norm of the float difference
// (Particle.cpp:222-224, measure.hpp:188-196). Called only inside a narrow band around the
// cutoff, where the FP32 squared distance cannot decide.
__device__ __noinline__ bool na_exact_in(float4 a, float4 b, float cutoff, bool nonzero)
{
    const double ax = __dsub_rn(static_cast<double>(a.x), static_cast<double>(b.x));
    const double ay = __dsub_rn(static_cast<double>(a.y), static_cast<double>(b.y));
    const double az = __dsub_rn(static_cast<double>(a.z), static_cast<double>(b.z));
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az));
    if (!(__dsqrt_rn(s) < static_cast<double>(cutoff)))
        return false;
    const double fx = static_cast<double>(__fsub_rn(b.x, a.x));
    const double fy = static_cast<double>(__fsub_rn(b.y, a.y));
    const double fz = static_cast<double>(__fsub_rn(b.z, a.z));
    double nrm = 0.0;
    if (!(fabs(fx) < 1e-40 && fabs(fy) < 1e-40 && fabs(fz) < 1e-40))
        nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy)), __dmul_rn(fz, fz)));
    const float d = __double2float_rn(nrm);
    return d < cutoff && (!nonzero || d != 0.0f);
}

__device__ __forceinline__ bool na_in(float r2, float lo2, float hi2, float4 a, float4 b, float cutoff,
                                      bool nonzero)
{
    if (r2 >= hi2)
        return false;
    if (r2 < lo2 && r2 > 1e-20f)
        return true;
    return na_exact_in(a, b, cutoff, nonzero);
}

// Packs the caller's arrays into the scratch: per-particle steric factors of the combination
// rules (CombinationRules.hpp:18-31), so that a pair needs products only: Amber and Lewitt use
// sqrt(eps_i eps_j) (r_i r_j)^(k/2), P = sqrt(eps) r^3, F = sqrt(eps) r^6 (Amber) or r^4
// (Lewitt); Zacharias uses eps_i eps_j (r_i r_j)^k, P = eps r^6, F = eps r^8.
__global__ void __launch_bounds__(256) k_na_pack(NaParams p, const float *__restrict__ xyz,
                                                 const float *__restrict__ radius,
                                                 const float *__restrict__ epsilon,
                                                 const float *__restrict__ charge,
                                                 const float *__restrict__ hydro,
                                                 const uint8_t *__restrict__ is_static, NaBuffers b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    const double r = radius ? static_cast<double>(radius[i]) : 0.0;
    const double e = epsilon ? static_cast<double>(epsilon[i]) : 0.0;
    double P = r, F = 0.0;
    if (p.steric_mode == BS_STERIC_LJ_12_6_AMBER || p.steric_mode == BS_STERIC_LJ_8_6_LEWITT)
    {
        const double se = sqrt(e), r2 = r * r;
        P = se * r2 * r;
        F = p.steric_mode == BS_STERIC_LJ_12_6_AMBER ? se * (r2 * r2 * r2) : se * (r2 * r2);
    }
    else if (p.steric_mode == BS_STERIC_LJ_8_6_ZACHARIAS)
    {
        const double r2 = r * r, r6 = r2 * r2 * r2;
        P = e * r6;
        F = e * (r6 * r2);
    }
    const float q = charge ? charge[i] : 0.0f;
    const float h = hydro ? hydro[i] : 0.0f;
    unsigned int fl = 0u;
    if (is_static && is_static[i])
        fl |= PF_STATIC;
    if (q != 0.0f)
        fl |= PF_CHARGED;
    if (h != 0.0f)
        fl |= PF_HYDROPHOBIC;
    b.pos[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], static_cast<float>(P));
    b.prm[i] = make_float4(static_cast<float>(F), q, h, __uint_as_float(fl));
}

// One thread per particle i; all particles j stream through shared memory in tiles of
// kNaBlock. Energies: FP32 per thread, FP64 per block, summed in block order by the last block.
__global__ void __launch_bounds__(kNaBlock) k_na_forces(NaParams p, float *__restrict__ forces,
                                                        double *__restrict__ energies, NaBuffers b)
{
    __shared__ float4 sh_pos[kNaBlock];
    __shared__ float4 sh_prm[kNaBlock];
    __shared__ double sh_e[kNaBlock / 32][kNaTerms];
    __shared__ bool last;
    const int i = blockIdx.x * kNaBlock + threadIdx.x;
    const bool valid = i < p.n;
    const float4 pi = valid ? b.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 qi = valid ? b.prm[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned int fi = __float_as_uint(qi.w);
    const bool dyn = valid && !(fi & PF_STATIC);
    const bool do_s = dyn && p.steric_on;
    const bool do_c = dyn && p.coulomb_on && (fi & PF_CHARGED);
    const bool do_h = dyn && p.hydro_on && (fi & PF_HYDROPHOBIC);
    float sx = 0.f, sy = 0.f, sz = 0.f, es = 0.f; // steric
    float cx = 0.f, cy = 0.f, cz = 0.f, ec = 0.f; // Coulomb
    float hx = 0.f, hy = 0.f, hz = 0.f, eh = 0.f; // hydrophobic
    for (int t0 = 0; t0 < p.n; t0 += kNaBlock)
    {
        const int jl = t0 + threadIdx.x;
        __syncthreads();
        if (jl < p.n)
        {
            sh_pos[threadIdx.x] = b.pos[jl];
            sh_prm[threadIdx.x] = b.prm[jl];
        }
        __syncthreads();
        const int m = min(kNaBlock, p.n - t0);
        if (!(do_s || do_c || do_h))
            continue;
        for (int k = 0; k < m; ++k)
        {
            const int j = t0 + k;
            if (j == i)
                continue;
            const float4 pj = sh_pos[k];
            const float4 qj = sh_prm[k];
            const unsigned int fj = __float_as_uint(qj.w);
            const float w = (fj & PF_STATIC) ? 1.0f : 0.5f;
            const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (do_s && na_in(r2, p.lo2_s, p.hi2_s, pi, pj, p.c_steric, false))
            {
                if (p.steric_mode == BS_STERIC_LINEAR)
                {
                    // E = (d - (ri + rj))^2 / 2 when overlapping, |F| = |d - (ri + rj)|
                    const float d = sqrtf(r2);
                    const float dv = d - (pi.w + pj.w);
                    if (dv <= 0.0f)
                    {
                        const float fod = d > 0.0f ? dv / d : 0.0f;
                        es = fmaf(w * 0.5f, dv * dv, es);
                        sx = fmaf(dx, fod, sx);
                        sy = fmaf(dy, fod, sy);
                        sz = fmaf(dz, fod, sz);
                    }
                }
                else if (r2 >= 0.01f) // d < 0.1 A gives zero
                {
                    const float inv2 = 1.0f / r2;
                    const float i6 = inv2 * inv2 * inv2;
                    const float t6 = pi.w * pj.w * i6;
                    float fod;
                    if (p.steric_mode == BS_STERIC_LJ_12_6_AMBER)
                    {
                        const float t12 = qi.x * qj.x * i6 * i6;
                        es = fmaf(w, t12 - 2.0f * t6, es);
                        fod = 12.0f * (t6 - t12) * inv2;
                    }
                    else if (p.steric_mode == BS_STERIC_LJ_8_6_LEWITT)
                    {
                        const float t8 = qi.x * qj.x * i6 * inv2;
                        es = fmaf(w, 3.0f * t8 - 4.0f * t6, es);
                        fod = 24.0f * (t6 - t8) * inv2;
                    }
                    else
                    {
                        const float t8 = qi.x * qj.x * i6 * inv2;
                        es = fmaf(w, t8 - t6, es);
                        fod = (6.0f * t6 - 8.0f * t8) * inv2;
                    }
                    sx = fmaf(dx, fod, sx);
                    sy = fmaf(dy, fod, sy);
                    sz = fmaf(dz, fod, sz);
                }
            }
            if (do_c && (fj & PF_CHARGED) && r2 >= 1e-6f && na_in(r2, p.lo2_c, p.hi2_c, pi, pj, p.c_coulomb, true))
            {
                const float inv = 1.0f / sqrtf(r2);
                float tq = qi.y * qj.y * inv;
                float fod;
                if (p.dist_dielectric)
                {
                    tq *= inv;
                    fod = -2.0f * tq * inv * inv;
                }
                else
                    fod = -tq * inv * inv;
                ec = fmaf(w, tq, ec);
                cx = fmaf(dx, fod, cx);
                cy = fmaf(dy, fod, cy);
                cz = fmaf(dz, fod, cz);
            }
            if (do_h && (fj & PF_HYDROPHOBIC) && na_in(r2, p.lo2_h, p.hi2_h, pi, pj, p.c_hydro, true))
            {
                const float d = sqrtf(r2);
                const float x = qi.z * qj.z * expf(-d);
                const float fod = x / d;
                eh = fmaf(-w, x, eh);
                hx = fmaf(dx, fod, hx);
                hy = fmaf(dy, fod, hy);
                hz = fmaf(dz, fod, hz);
            }
        }
    }
    if (valid)
    {
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (dyn)
        {
            fx = sx * p.kf_steric + cx * p.kf_elec + hx * p.kf_hydro;
            fy = sy * p.kf_steric + cy * p.kf_elec + hy * p.kf_hydro;
            fz = sz * p.kf_steric + cz * p.kf_elec + hz * p.kf_hydro;
        }
        forces[3 * i] = fx;
        forces[3 * i + 1] = fy;
        forces[3 * i + 2] = fz;
    }
    // ---- energies: warp sums in FP32, block and grid sums in FP64, fixed order ----
    float e[kNaTerms] = {es * p.ke_steric, ec * p.ke_elec, eh * p.ke_hydro};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kNaTerms; ++q)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            e[q] += __shfl_down_sync(0xffffffffu, e[q], o);
        if (lane == 0)
            sh_e[wid][q] = static_cast<double>(e[q]);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int q = 0; q < kNaTerms; ++q)
        {
            double s = 0.0;
            for (int w = 0; w < kNaBlock / 32; ++w)
                s += sh_e[w][q];
            b.blk[blockIdx.x * kNaTerms + q] = s;
        }
        __threadfence();
        last = atomicAdd(b.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0)
        return;
    __threadfence();
    double tot[kNaTerms] = {0.0, 0.0, 0.0};
    for (unsigned int k = 0; k < gridDim.x; ++k)
#pragma unroll
        for (int q = 0; q < kNaTerms; ++q)
            tot[q] += *(volatile double *)&b.blk[k * kNaTerms + q];
    for (int q = 0; q < BS_NUM_ENERGIES; ++q)
        energies[q] = 0.0;
    energies[BS_ENERGY_STERIC] = tot[0];
    energies[BS_ENERGY_ELECTROSTATIC] = tot[1];
    energies[BS_ENERGY_HYDROPHOBIC] = tot[2];
    *b.done = 0u; // ready for the next call
}

float na_band_lo2(double c) { return static_cast<float>((c * (1.0 - 1.0 / 16384.0)) * (c * (1.0 - 1.0 / 16384.0))); }
float na_band_hi2(double c) { return static_cast<float>((c * (1.0 + 1.0 / 16384.0)) * (c * (1.0 + 1.0 / 16384.0))); }

void na_message(char *err, size_t len, const char *msg)
{
    if (err && len)
    {
        std::strncpy(err, msg, len - 1);
        err[len - 1] = '\0';
    }
}

// Scratch address per device, looked up once with that device current.
constexpr int kNaMaxDevices = 64;
std::mutex na_mutex;
unsigned char *na_ptr[kNaMaxDevices] = {};

} // namespace
} // namespace bsg

using namespace bsg;

extern "C" int bs_nonbonded_forces_noalloc(const bs_config *cfg, int64_t n, const float *d_xyz,
                                           const float *d_radius, const float *d_epsilon,
                                           const float *d_charge, const float *d_hydrophobicity,
                                           const uint8_t *d_is_static, float *d_forces, double *d_energies,
                                           void *stream, char *err, size_t err_len)
{
    char msg[192];
    if (!cfg || !d_xyz || !d_forces || !d_energies)
    {
        na_message(err, err_len, "null argument: cfg, xyz, forces and energies are required");
        return BS_E_ARG;
    }
    if (n < 1 || n > kNaMaxN)
    {
        std::snprintf(msg, sizeof msg, "particle count %lld outside [1, %d], the size of the static scratch",
                      static_cast<long long>(n), kNaMaxN);
        na_message(err, err_len, msg);
        return BS_E_ARG;
    }
    if (cfg->steric_enable)
    {
        if (!(cfg->steric_cutoff > 0.0))
        {
            na_message(err, err_len, "Steric cutoff must be > 0");
            return BS_E_ARG;
        }
        if (cfg->steric_mode < BS_STERIC_LINEAR || cfg->steric_mode > BS_STERIC_LJ_8_6_ZACHARIAS)
        {
            na_message(err, err_len, "unknown steric mode");
            return BS_E_ARG;
        }
        if (!d_radius || (cfg->steric_mode != BS_STERIC_LINEAR && !d_epsilon))
        {
            na_message(err, err_len, "steric term needs radius (and epsilon in the Lennard-Jones modes)");
            return BS_E_ARG;
        }
    }
    if (cfg->coulomb_enable && !(cfg->coulomb_cutoff > 0.0))
    {
        na_message(err, err_len, "Coulomb cutoff must be > 0");
        return BS_E_ARG;
    }
    if (cfg->coulomb_enable && !(cfg->coulomb_dielectric > 0.0))
    {
        na_message(err, err_len, "Coulomb dielectric must be > 0");
        return BS_E_ARG;
    }
    if (cfg->hydrophobicity_enable && !(cfg->hydrophobicity_cutoff > 0.0))
    {
        na_message(err, err_len, "Hydrophobicity cutoff must be > 0");
        return BS_E_ARG;
    }

    // Set-up, once per device: resolve the scratch address with that device current and clear
    // the block counter. The first call on a device does this (it loads this module onto the
    // device), so it should come before any stream capture.
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess || dev < 0 || dev >= kNaMaxDevices)
    {
        std::snprintf(msg, sizeof msg, "no usable current device (%s)", cudaGetErrorString(rc));
        na_message(err, err_len, msg);
        return BS_E_CUDA;
    }
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(na_mutex);
        if (!na_ptr[dev])
        {
            void *ptr = nullptr;
            rc = cudaGetSymbolAddress(&ptr, na_scratch);
            if (rc != cudaSuccess)
            {
                std::snprintf(msg, sizeof msg, "cudaGetSymbolAddress of the scratch failed: %s",
                              cudaGetErrorString(rc));
                na_message(err, err_len, msg);
                return BS_E_CUDA;
            }
            rc = cudaMemset(static_cast<unsigned char *>(ptr) + kNaDoneOff, 0, sizeof(unsigned int));
            if (rc == cudaSuccess)
                rc = cudaDeviceSynchronize();
            if (rc != cudaSuccess)
            {
                std::snprintf(msg, sizeof msg, "clearing the scratch counter failed: %s", cudaGetErrorString(rc));
                na_message(err, err_len, msg);
                return BS_E_CUDA;
            }
            na_ptr[dev] = static_cast<unsigned char *>(ptr);
        }
        base = na_ptr[dev];
    }

    NaParams p{};
    p.n = static_cast<int>(n);
    p.steric_on = cfg->steric_enable != 0;
    p.coulomb_on = cfg->coulomb_enable != 0 && d_charge != nullptr;
    p.hydro_on = cfg->hydrophobicity_enable != 0 && d_hydrophobicity != nullptr;
    p.steric_mode = cfg->steric_mode;
    p.dist_dielectric = cfg->dielectric_mode == BS_DIELECTRIC_DISTANCE;
    p.c_steric = static_cast<float>(cfg->steric_cutoff);
    p.c_coulomb = static_cast<float>(cfg->coulomb_cutoff);
    p.c_hydro = static_cast<float>(cfg->hydrophobicity_cutoff);
    p.lo2_s = na_band_lo2(p.c_steric);
    p.hi2_s = na_band_hi2(p.c_steric);
    p.lo2_c = na_band_lo2(p.c_coulomb);
    p.hi2_c = na_band_hi2(p.c_coulomb);
    p.lo2_h = na_band_lo2(p.c_hydro);
    p.hi2_h = na_band_hi2(p.c_hydro);
    const float kspring = static_cast<float>(kSpringForceConvert);
    p.kf_steric = kspring * static_cast<float>(cfg->steric_gridscale);
    p.ke_steric = static_cast<float>(cfg->steric_gridscale);
    const double D = cfg->coulomb_dielectric > 0.0 ? cfg->coulomb_dielectric : 1.0;
    p.kf_elec = static_cast<float>(kElecForceConvert / (4.0 * kPi) * cfg->coulomb_scale / D);
    p.ke_elec = static_cast<float>(kCoulombEnergyPerA * cfg->coulomb_scale / D);
    p.kf_hydro = kspring * static_cast<float>(cfg->hydrophobicity_scale);
    p.ke_hydro = static_cast<float>(kAvogadro * 1.0E-3) * static_cast<float>(cfg->hydrophobicity_scale);

    const NaBuffers b = na_buffers(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_na_pack<<<(p.n + 255) / 256, 256, 0, st>>>(p, d_xyz, d_radius, d_epsilon, d_charge, d_hydrophobicity,
                                                  d_is_static, b);
    k_na_forces<<<(p.n + kNaBlock - 1) / kNaBlock, kNaBlock, 0, st>>>(p, d_forces, d_energies, b);
    rc = cudaGetLastError();
    if (rc != cudaSuccess)
    {
        std::snprintf(msg, sizeof msg, "kernel launch failed: %s", cudaGetErrorString(rc));
        na_message(err, err_len, msg);
        return BS_E_CUDA;
    }
    return BS_OK;
}
