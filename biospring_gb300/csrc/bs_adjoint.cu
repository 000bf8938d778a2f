// bs_adjoint.cu -- discrete adjoint of the damped step, for gradients of a loss on the final
// positions with respect to every spring's stiffness and rest length, and every particle's charge.
//
// The step being differentiated is the one the forward kernels integrate (Particle.cpp:80-84,
// 109-128; SpringNetwork.cpp:63-198): with F_i(x) the conservative force on particle i,
//     v' = a_i v + b_i F_i(x),   a_i = 1 - gamma dt / m_i (1 without viscosity),  b_i = dt / m_i
//     x' = x + dt v'
// (a_i = 1, b_i = 0 for m_i <= 0 and for static particles, which never move). For the loss
// L(x_N) the adjoints lambda_x = dL/dx_n and lambda_v = dL/dv_n run backwards:
//     mu      = lambda_v' + dt lambda_x'          (adjoint of v')
//     nu_i    = b_i mu_i
//     lambda_x = lambda_x' + sum_j H_ij (nu_j - nu_i)
//     lambda_v = a_i mu_i
//     dL/dtheta += sum_i nu_i . dF_i/dtheta
// where, for a central pair force F_i = phi(d) u (u = (x_j - x_i) / d),
//     H w = phi'(d) (u.w) u + phi(d) / d (w - (u.w) u).
// Springs (spring.hpp:17-29): phi = C s k (d - r0), phi' = C s k, dF_i/dk = C s (d - r0) u,
// dF_i/dr0 = -C s k u. Linear steric overlap (steric.hpp:37-59): phi = C s' (d - (r_i + r_j)) when
// d < r_i + r_j and the pair is within the cutoff, phi' = C s'. Coulomb (electrostatic.hpp:16-49):
// phi = -C q_i q_j / d^2 (or -2 C q_i q_j / d^3 with eps = D r), dF_i/dq_i = (phi / q_i) u.
//
// Each directed spring entry (the spring seen from one end) owns two gradient accumulators, so
// the sums need no atomics and are deterministic; the two ends are added at the end.
//
// The stretch d - r0 enters dL/dk and phi directly, and near rest it is far smaller than d: in
// plain FP32 it would carry the rounding of d (1e-7 relative to d, i.e. often several percent
// of d - r0). It is formed as (d^2 - r0^2) / (d + r0) with d^2 and r0^2 in float-float, from the
// separation in float-float (positions plus their remainders when they are carried).

#include "bs_device.cuh"

namespace bsg
{
namespace
{

// H w of one central pair force.
__device__ __forceinline__ void hvp(float phi, float dphi, float inv, float ux, float uy, float uz, float wx, float wy,
                                    float wz, float &hx, float &hy, float &hz)
{
    const float uw = ux * wx + uy * wy + uz * wz;
    const float a = phi * inv;       // phi / d
    const float c = (dphi - a) * uw; // (phi' - phi / d) (u.w)
    hx = fmaf(a, wx, fmaf(c, ux, hx));
    hy = fmaf(a, wy, fmaf(c, uy, hy));
    hz = fmaf(a, wz, fmaf(c, uz, hz));
}

// Coulomb pairs of slot s (list 1), lane t of T: the Hessian term of pairs of two charges, and
// this step's dL/dq terms when charge gradients are asked for. With F_s = phi u, u = (x_j - x_s)/d,
// phi = -C q_s q_j / d^2 (constant dielectric; -2 C q_s q_j / d^3 with eps = D r) and C the
// device's Coulomb constant: dL/dq_s += (phi / q_s) u.(nu_s - nu_j), and the same with phi / q_j for
// a static partner, which has no row of its own (added atomically). The rows list every partner
// of the slot when charge gradients are asked for, so uncharged particles get theirs too.
template <int T>
__device__ __forceinline__ void adj_coulomb(const Params &p, const AdjState &a, int s, int t, int lb, float4 xi,
                                            float4 ni, float qs, float &hx, float &hy, float &hz, float &gqs)
{
    const PairList &L = p.pl[1];
    const int cnt = L.cnt[s];
    const size_t row = static_cast<size_t>(s) * L.cap;
    const float C = p.k_elec_f;
    const bool dist = p.dielectric_mode == BS_DIELECTRIC_DISTANCE;
    for (int k = t; k < cnt; k += T)
    {
        const unsigned int e = L.idx[row + k];
        const int j = static_cast<int>(e & kSlotMask);
        const bool st = (e & kEntryStatic) != 0;
        const float4 xj = a.x[j];
        const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!pair_in(r2, p.lo2_c, p.hi2_c, xi, xj, p.c_coulomb, true) || r2 < 1e-6f)
            continue;
        const float qj = p.chg[lb][j];
        if (qs == 0.0f && qj == 0.0f)
            continue;
        const float inv = rsqrt_nr(r2);
        const float inv2 = inv * inv;
        const float per_s = dist ? -2.0f * C * qj * inv2 * inv : -C * qj * inv2;
        const float per_j = dist ? -2.0f * C * qs * inv2 * inv : -C * qs * inv2;
        const float phi = per_s * qs;
        const float dphi = (dist ? -3.0f : -2.0f) * phi * inv;
        const float ux = dx * inv, uy = dy * inv, uz = dz * inv;
        const float4 nj = st ? make_float4(0.f, 0.f, 0.f, 0.f) : a.nu_in[j];
        if (phi != 0.0f)
            hvp(phi, dphi, inv, ux, uy, uz, nj.x - ni.x, nj.y - ni.y, nj.z - ni.z, hx, hy, hz);
        if (a.gq)
        {
            const float un = ux * (ni.x - nj.x) + uy * (ni.y - nj.y) + uz * (ni.z - nj.z);
            gqs = fmaf(per_s, un, gqs);
            if (st)
                atomicAdd(&a.gq[p.perm[lb][j]], per_j * un);
        }
    }
}

// Separation xj - xi as float-float per axis, squared length r2 = (r2h, r2l), and the stretch
// d - r0 accurate to a few ulps of itself. Returns false for coincident particles.
__device__ __forceinline__ bool spring_geometry(float4 xi, float4 xj, float4 li, float4 lj, float r0, float &dx,
                                                float &dy, float &dz, float &d, float &inv, float &stretch)
{
    float hx, ex, hy, ey, hz, ez;
    two_sum(xj.x, -xi.x, hx, ex);
    two_sum(xj.y, -xi.y, hy, ey);
    two_sum(xj.z, -xi.z, hz, ez);
    ex += lj.x - li.x;
    ey += lj.y - li.y;
    ez += lj.z - li.z;
    float r2h = 0.0f, r2l = 0.0f;
    const float h3[3] = {hx, hy, hz}, e3[3] = {ex, ey, ez};
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const float ph = h3[c] * h3[c];
        const float pl = fmaf(h3[c], h3[c], -ph) + 2.0f * h3[c] * e3[c];
        ff_add(r2h, r2l, ph, pl);
    }
    if (!(r2h > 0.0f))
        return false;
    dx = hx + ex;
    dy = hy + ey;
    dz = hz + ez;
    inv = rsqrt_nr(r2h);
    d = r2h * inv;
    const float q = r0 * r0, ql = fmaf(r0, r0, -q);
    float nh, ne;
    two_sum(r2h, -q, nh, ne);
    ne += r2l - ql;
    stretch = (nh + ne) / (d + r0);
    return true;
}

// Linear steric overlaps of slot s from one pair list, lane t of T.
template <int T, int KIND>
__device__ __forceinline__ void adj_steric(const Params &p, const AdjState &a, int s, int t, float4 xi, float4 ni,
                                           float &hx, float &hy, float &hz)
{
    const PairList &L = p.pl[KIND == 2 ? kListStericStatic : 0];
    const int cnt = L.cnt[s];
    const size_t row = static_cast<size_t>(s) * L.cap;
    const float cs = p.k_spring_f * p.steric_scale;
    for (int k = t; k < cnt; k += T)
    {
        int j;
        if (KIND == 0)
            j = s + static_cast<int>(reinterpret_cast<const short *>(L.idx)[row + k]);
        else
            j = static_cast<int>(L.idx[row + k] & kSlotMask);
        const float4 xj = a.x[j];
        const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!pair_in(r2, p.lo2_s, p.hi2_s, xi, xj, p.c_steric, false) || !(r2 > 0.0f))
            continue;
        const float d = sqrtf(r2);
        const float dv = d - (xi.w + xj.w);
        if (dv > 0.0f)
            continue;
        const float inv = 1.0f / d;
        const float4 nj = KIND == 2 ? make_float4(0.f, 0.f, 0.f, 0.f) : a.nu_in[j];
        hvp(cs * dv, cs, inv, dx * inv, dy * inv, dz * inv, nj.x - ni.x, nj.y - ni.y, nj.z - ni.z, hx, hy, hz);
    }
}

// One backward step for every particle: reads nu of step n+1 and the positions at the start of
// step n, updates lambda_x and lambda_v in place, writes nu of step n, and adds this step's
// terms to the per-entry spring gradients. T lanes per particle, as in the forward step.
template <int T>
__global__ void __launch_bounds__(kStepBlock) k_adj_step(Params p, AdjState a)
{
    const Ctl *ctl = p.ctl;
    const int lb = ctl->lbuf;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = g / T, t = g % T;
    const bool lead = t == 0;
    const unsigned int fi = s < p.n ? p.flags[lb][s] : PF_STATIC;
    const bool active = s < p.n && !(fi & PF_STATIC);
    float hx = 0.f, hy = 0.f, hz = 0.f, gqs = 0.f;
    float4 xi = make_float4(0.f, 0.f, 0.f, 0.f), ni = xi, li = xi;
    if (active)
    {
        xi = a.x[s];
        ni = a.nu_in[s];
        if (a.xlo)
            li = a.xlo[s];
        if (p.spring_on)
        {
            const int deg = p.se_deg[s];
            const size_t stride = static_cast<size_t>(p.npad);
            const float cs = p.k_spring_f * p.spring_scale;
            for (int k = t; k < deg; k += T)
            {
                // the entry's table fields and its gradient accumulators are read together, before
                // the partner's state, so the accumulators do not wait behind the partner loads
                const size_t at = static_cast<size_t>(k) * stride + s;
                const unsigned int c = p.se_col[at];
                const float kk = p.se_k[at], r0 = p.se_r0[at];
                const unsigned int sid = p.se_sid[at];
                const float gk = a.gk[sid], gr0 = a.gr0[sid];
                if (c & kEntryInactive)
                    continue;
                const int j = static_cast<int>(c & kSlotMask);
                const float4 xj = a.x[j];
                const float4 lj = a.xlo ? a.xlo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 nj = (c & kEntryStatic) ? make_float4(0.f, 0.f, 0.f, 0.f) : a.nu_in[j];
                float dx, dy, dz, d, inv, dv;
                if (!spring_geometry(xi, xj, li, lj, r0, dx, dy, dz, d, inv, dv))
                    continue;
                const float ux = dx * inv, uy = dy * inv, uz = dz * inv;
                hvp(cs * kk * dv, cs * kk, inv, ux, uy, uz, nj.x - ni.x, nj.y - ni.y, nj.z - ni.z, hx, hy, hz);
                const float un = ux * ni.x + uy * ni.y + uz * ni.z;
                a.gk[sid] = gk + cs * dv * un;
                a.gr0[sid] = gr0 - cs * kk * un;
            }
        }
        if (p.steric_on)
        {
            if (p.pl16)
                adj_steric<T, 0>(p, a, s, t, xi, ni, hx, hy, hz);
            else
                adj_steric<T, 1>(p, a, s, t, xi, ni, hx, hy, hz);
            if (p.pl[kListStericStatic].on && p.pl[kListStericStatic].cnt[s] > 0)
                adj_steric<T, 2>(p, a, s, t, xi, ni, hx, hy, hz);
        }
        if (p.coulomb_on)
            adj_coulomb<T>(p, a, s, t, lb, xi, ni, p.chg[lb][s], hx, hy, hz, gqs);
    }
    if (T > 1)
    {
        hx = group_sum<T>(hx);
        hy = group_sum<T>(hy);
        hz = group_sum<T>(hz);
        if (a.gq)
            gqs = group_sum<T>(gqs);
    }
    if (!lead || s >= p.npad)
        return;
    if (!active)
    {
        a.nu_out[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (a.gq && p.coulomb_on)
        a.gq[p.perm[lb][s]] += gqs;
    const float m = p.iprm[lb][s].x;
    const float b = m > 0.0f ? p.dt / m : 0.0f;
    const float av = (m > 0.0f && p.visc_on) ? 1.0f - p.visc * p.dt / m : 1.0f;
    const float4 lx = a.lx[s], lv = a.lv[s];
    const float mux = fmaf(p.dt, lx.x, lv.x), muy = fmaf(p.dt, lx.y, lv.y), muz = fmaf(p.dt, lx.z, lv.z);
    const float nlx = lx.x + hx, nly = lx.y + hy, nlz = lx.z + hz;
    const float nvx = av * mux, nvy = av * muy, nvz = av * muz;
    a.lx[s] = make_float4(nlx, nly, nlz, 0.f);
    a.lv[s] = make_float4(nvx, nvy, nvz, 0.f);
    a.nu_out[s] = make_float4(b * fmaf(p.dt, nlx, nvx), b * fmaf(p.dt, nly, nvy), b * fmaf(p.dt, nlz, nvz), 0.f);
}

// Loss L = (1/n) sum_i |x_i - target_i|^2 at the current state (all particles), and the adjoint
// state at the final step: lambda_x = 2 (x - target) / n, lambda_v = 0, nu = b dt lambda_x
// (zero for static particles). Per-block partial sums in FP64; the last block writes the total.
__global__ void __launch_bounds__(256) k_adj_init(Params p, AdjState a, const float4 *target, double *blk,
                                                  unsigned int *done, double *loss)
{
    const Ctl *ctl = p.ctl;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (s < p.npad)
    {
        float4 lx = make_float4(0.f, 0.f, 0.f, 0.f), nu = lx;
        if (s < p.n)
        {
            const int id = p.perm[lb][s];
            const float4 x = p.pos[sb][s], tg = target[id];
            float dx = x.x - tg.x, dy = x.y - tg.y, dz = x.z - tg.z;
            if (p.pos_lo[0])
            {
                const float4 lo = p.pos_lo[sb][s];
                dx += lo.x;
                dy += lo.y;
                dz += lo.z;
            }
            l = static_cast<double>(dx) * dx + static_cast<double>(dy) * dy + static_cast<double>(dz) * dz;
            if (!(p.flags[lb][s] & PF_STATIC))
            {
                const float c = 2.0f / static_cast<float>(p.n);
                lx = make_float4(c * dx, c * dy, c * dz, 0.f);
                const float m = p.iprm[lb][s].x;
                const float b = m > 0.0f ? p.dt / m : 0.0f;
                nu = make_float4(b * p.dt * lx.x, b * p.dt * lx.y, b * p.dt * lx.z, 0.f);
            }
        }
        a.lx[s] = lx;
        a.lv[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.nu_in[s] = nu;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = l;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o)
            sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0)
    {
        blk[blockIdx.x] = sh[0];
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0)
    {
        __threadfence();
        double tot = 0.0;
        for (unsigned int b = 0; b < gridDim.x; ++b)
            tot += __ldcg(&blk[b]);
        *loss = tot / static_cast<double>(p.n);
        *done = 0u;
    }
}

// lambda_x, lambda_v of the current layout -> caller order (dir = 0), or back, recomputing nu
// (dir = 1).
__global__ void k_adj_permute(Params p, AdjState a, float4 *cx, float4 *cv, int dir)
{
    const Ctl *ctl = p.ctl;
    const int lb = ctl->lbuf;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.npad)
        return;
    if (s >= p.n)
    {
        if (dir == 1)
        {
            a.lx[s] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.lv[s] = a.lx[s];
            a.nu_in[s] = a.lx[s];
        }
        return;
    }
    const int id = p.perm[lb][s];
    if (dir == 0)
    {
        cx[id] = a.lx[s];
        cv[id] = a.lv[s];
        return;
    }
    const float4 lx = cx[id], lv = cv[id];
    a.lx[s] = lx;
    a.lv[s] = lv;
    float4 nu = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!(p.flags[lb][s] & PF_STATIC))
    {
        const float m = p.iprm[lb][s].x;
        const float b = m > 0.0f ? p.dt / m : 0.0f;
        nu = make_float4(b * fmaf(p.dt, lx.x, lv.x), b * fmaf(p.dt, lx.y, lv.y), b * fmaf(p.dt, lx.z, lv.z), 0.f);
    }
    a.nu_in[s] = nu;
}

// Positions at the start of the next step (current buffer) -> dst, and their remainders -> dst_lo
// when positions carry them.
__global__ void k_adj_save(Params p, float4 *dst, float4 *dst_lo)
{
    const Ctl *ctl = p.ctl;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.npad)
        return;
    dst[s] = p.pos[ctl->sbuf][s];
    if (dst_lo && p.pos_lo[0])
        dst_lo[s] = p.pos_lo[ctl->sbuf][s];
}

// dL/dk and dL/dr0 of every spring: the sum of its two directed entries.
__global__ void k_adj_combine(int nsp, const float *gk, const float *gr0, float *ok, float *or0)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsp)
        return;
    ok[t] = gk[2 * t] + gk[2 * t + 1];
    or0[t] = gr0[2 * t] + gr0[2 * t + 1];
}

} // namespace

int launch_adj_step(const Params &p, const AdjState &a, cudaStream_t st)
{
    // Lanes per particle: a backward step does about twice the forward's work per spring and
    // pair (Hessian-vector products, gradient sums) on a grid of the same size, so small systems
    // take 16 lanes (10,000 particles: 160,000 threads, 8 blocks of 128 per SM) to keep enough
    // loads in flight (32 lanes: 10% slower); larger ones follow the forward step.
    const int T = p.n < 20000 ? 16 : (p.step_lanes >= 8 ? 8 : (p.step_lanes == 2 ? 2 : 4));
    const int nb = static_cast<int>((static_cast<long long>(p.npad) * T + kStepBlock - 1) / kStepBlock);
    if (T == 16)
        k_adj_step<16><<<nb, kStepBlock, 0, st>>>(p, a);
    else if (T == 8)
        k_adj_step<8><<<nb, kStepBlock, 0, st>>>(p, a);
    else if (T == 2)
        k_adj_step<2><<<nb, kStepBlock, 0, st>>>(p, a);
    else
        k_adj_step<4><<<nb, kStepBlock, 0, st>>>(p, a);
    return 1;
}

int launch_adj_init(const Params &p, const AdjState &a, const float4 *target, double *blk, unsigned int *done,
                    double *loss, cudaStream_t st)
{
    k_adj_init<<<(p.npad + 255) / 256, 256, 0, st>>>(p, a, target, blk, done, loss);
    return 1;
}

int launch_adj_permute(const Params &p, const AdjState &a, float4 *cx, float4 *cv, int dir, cudaStream_t st)
{
    k_adj_permute<<<(p.npad + 255) / 256, 256, 0, st>>>(p, a, cx, cv, dir);
    return 1;
}

int launch_adj_save(const Params &p, float4 *dst, float4 *dst_lo, cudaStream_t st)
{
    k_adj_save<<<(p.npad + 255) / 256, 256, 0, st>>>(p, dst, dst_lo);
    return 1;
}

int launch_adj_combine(int nsp, const float *gk, const float *gr0, float *ok, float *or0, cudaStream_t st)
{
    if (nsp > 0)
        k_adj_combine<<<(nsp + 255) / 256, 256, 0, st>>>(nsp, gk, gr0, ok, or0);
    return 1;
}

} // namespace bsg
