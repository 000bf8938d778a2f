// bs_rigid.cu -- rigid-body dynamics of the step (RigidBodiesManager::SolveRigidBodiesDynamic,
// src/rigidbody/RigidBodiesManager.cpp:45-60).
//
// The step kernel leaves the total force of every rigid particle (springs to non-rigid partners,
// nonbonded terms, viscosity, IMPALA, external force) in rforce and does not move it. Then one
// block per body:
//   1. sums the force and the torque (x_i - X) x f_i over the body's members
//      (RigidBody::computeParticleForceAndTorque, RigidBody.cpp:567-580) in float-float;
//   2. advances the body (RigidBody::solve, RigidBody.cpp:455-483): a = F / M, v += a dt,
//      X += v dt + a/2 dt^2, L += tau dt, omega = I^-1 L with the sphere inertia I = 2/5 M,
//      rotation by the quaternion (omega sin(|omega| dt / 2), cos(|omega| dt / 2)) (the axis is
//      omega itself, not normalised, as in the reference), renormalised;
//   3. places every member at X + q p0 q^-1 with velocity (new - old) / dt
//      (RigidBody::integrateParticleVelocity, RigidBody.cpp:600-635), p0 being the member's
//      offset from the barycentre at set-up, taken by its index within its own body.
// Float operations are written without contraction, in the reference's order, so a body
// follows the reference up to the order of the force sum.

#include "bs_device.cuh"

namespace bsg
{
namespace
{

constexpr int kRigidBlock = 256;

struct Quat
{
    float x, y, z, w;
};

// Quaternion product (Quaternion.cpp): vector part b.v a.w + a.v b.w + a.v x b.v.
__device__ __forceinline__ Quat qmul(Quat a, Quat b)
{
    const float cx = __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y));
    const float cy = __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z));
    const float cz = __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x));
    Quat r;
    r.x = __fadd_rn(__fadd_rn(__fmul_rn(b.x, a.w), __fmul_rn(a.x, b.w)), cx);
    r.y = __fadd_rn(__fadd_rn(__fmul_rn(b.y, a.w), __fmul_rn(a.y, b.w)), cy);
    r.z = __fadd_rn(__fadd_rn(__fmul_rn(b.z, a.w), __fmul_rn(a.z, b.w)), cz);
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
    r.w = __fsub_rn(__fmul_rn(a.w, b.w), dot);
    return r;
}

__device__ __forceinline__ float qnorm2(Quat q)
{
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.x, q.x), __fmul_rn(q.y, q.y)), __fmul_rn(q.z, q.z)),
                     __fmul_rn(q.w, q.w));
}

// Normalisation, skipped for a magnitude at or below 0.005 (Quaternion.cpp).
__device__ __forceinline__ Quat qnormalize(Quat q)
{
    const float m = __fsqrt_rn(qnorm2(q));
    if (m > 0.005f)
    {
        q.x = __fdiv_rn(q.x, m);
        q.y = __fdiv_rn(q.y, m);
        q.z = __fdiv_rn(q.z, m);
        q.w = __fdiv_rn(q.w, m);
    }
    return q;
}

// Inverse: conjugate over the squared magnitude (Quaternion.cpp).
__device__ __forceinline__ Quat qinverse(Quat q)
{
    const float wwxx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.w, q.w), __fmul_rn(q.x, q.x)), __fmul_rn(q.y, q.y)),
                                 __fmul_rn(q.z, q.z));
    float a = __fsqrt_rn(wwxx);
    a = __fmul_rn(a, a);
    a = __fdiv_rn(1.0f, a);
    Quat r;
    r.x = __fmul_rn(-q.x, a);
    r.y = __fmul_rn(-q.y, a);
    r.z = __fmul_rn(-q.z, a);
    r.w = __fmul_rn(q.w, a);
    return r;
}

__global__ void __launch_bounds__(kRigidBlock) k_rigid(Params p)
{
    Ctl *ctl = p.ctl;
    // the step kernel advances ctl->steps when it completes a step; bodies that already moved
    // for this step count (a status bit stopped the step kernel) stay
    const long long steps = *(volatile const long long *)&ctl->steps;
    if (steps == *(volatile const long long *)&ctl->rigid_steps)
        return;
    const int b = blockIdx.x;
    const int m0 = p.body_start[b], m1 = p.body_start[b + 1];
    const int snew = ctl->sbuf, sold = snew ^ 1, lb = ctl->lbuf;
    (void)lb;
    __shared__ BodyState sh_body;
    if (threadIdx.x == 0)
        sh_body = p.body[b];
    __syncthreads();
    const float X = sh_body.pos.x, Y = sh_body.pos.y, Z = sh_body.pos.z;

    // ---- 1. force and torque of the body ----
    float acc[6][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int m = m0 + threadIdx.x; m < m1; m += blockDim.x)
    {
        const int s = p.inv[p.body_ids[m]];
        const float4 f = p.rforce[s];
        const float4 x = p.pos[sold][s];
        const float rx = __fsub_rn(x.x, X), ry = __fsub_rn(x.y, Y), rz = __fsub_rn(x.z, Z);
        const float t[6] = {f.x, f.y, f.z, __fsub_rn(__fmul_rn(ry, f.z), __fmul_rn(rz, f.y)),
                            __fsub_rn(__fmul_rn(rz, f.x), __fmul_rn(rx, f.z)),
                            __fsub_rn(__fmul_rn(rx, f.y), __fmul_rn(ry, f.x))};
#pragma unroll
        for (int k = 0; k < 6; ++k)
            ff_add(acc[k][0], acc[k][1], t[k], 0.0f);
    }
    __shared__ float sh_acc[6][2][kRigidBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k)
    {
        float hi = acc[k][0], lo = acc[k][1];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
            const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
            ff_add(hi, lo, h2, l2);
        }
        if (lane == 0)
        {
            sh_acc[k][0][warp] = hi;
            sh_acc[k][1][warp] = lo;
        }
    }
    __syncthreads();

    // ---- 2. the body's step (thread 0) ----
    __shared__ Quat sh_q;
    __shared__ float sh_X[3];
    if (threadIdx.x == 0)
    {
        float tot[6];
        for (int k = 0; k < 6; ++k)
        {
            float hi = 0.f, lo = 0.f;
            for (int w = 0; w < kRigidBlock / 32; ++w)
                ff_add(hi, lo, sh_acc[k][0][w], sh_acc[k][1][w]);
            tot[k] = __fadd_rn(hi, lo);
        }
        BodyState bs = sh_body;
        const float dt = p.dt;
        const float M = static_cast<float>(bs.mass);
        const float ax = __fdiv_rn(tot[0], M), ay = __fdiv_rn(tot[1], M), az = __fdiv_rn(tot[2], M);
        bs.vel.x = __fadd_rn(bs.vel.x, __fmul_rn(ax, dt));
        bs.vel.y = __fadd_rn(bs.vel.y, __fmul_rn(ay, dt));
        bs.vel.z = __fadd_rn(bs.vel.z, __fmul_rn(az, dt));
        const float t1x = __fmul_rn(bs.vel.x, dt), t1y = __fmul_rn(bs.vel.y, dt), t1z = __fmul_rn(bs.vel.z, dt);
        const float t2x = __fmul_rn(__fmul_rn(__fmul_rn(ax, 0.5f), dt), dt);
        const float t2y = __fmul_rn(__fmul_rn(__fmul_rn(ay, 0.5f), dt), dt);
        const float t2z = __fmul_rn(__fmul_rn(__fmul_rn(az, 0.5f), dt), dt);
        bs.pos.x = __fadd_rn(bs.pos.x, __fadd_rn(t1x, t2x));
        bs.pos.y = __fadd_rn(bs.pos.y, __fadd_rn(t1y, t2y));
        bs.pos.z = __fadd_rn(bs.pos.z, __fadd_rn(t1z, t2z));
        bs.L.x = __fadd_rn(bs.L.x, __fmul_rn(tot[3], dt));
        bs.L.y = __fadd_rn(bs.L.y, __fmul_rn(tot[4], dt));
        bs.L.z = __fadd_rn(bs.L.z, __fmul_rn(tot[5], dt));
        const float ox = static_cast<float>(__dmul_rn(bs.ibodyinv, static_cast<double>(bs.L.x)));
        const float oy = static_cast<float>(__dmul_rn(bs.ibodyinv, static_cast<double>(bs.L.y)));
        const float oz = static_cast<float>(__dmul_rn(bs.ibodyinv, static_cast<double>(bs.L.z)));
        // |omega| as the reference's measure::norm: FP64 square root of the float components
        float nrm = 0.0f;
        if (!(fabsf(ox) < 1e-40f && fabsf(oy) < 1e-40f && fabsf(oz) < 1e-40f))
        {
            const double dx = ox, dy = oy, dz = oz;
            nrm = static_cast<float>(sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz))));
        }
        const float angle = static_cast<float>(__dmul_rn(static_cast<double>(nrm), static_cast<double>(dt)));
        const double half = static_cast<double>(angle) / 2.0;
        const float sa = static_cast<float>(sin(half));
        const float ca = static_cast<float>(cos(half));
        Quat dq{__fmul_rn(ox, sa), __fmul_rn(oy, sa), __fmul_rn(oz, sa), ca};
        dq = qnormalize(dq);
        Quat q{bs.q.x, bs.q.y, bs.q.z, bs.q.w};
        q = qnormalize(qmul(dq, q));
        bs.q = make_float4(q.x, q.y, q.z, q.w);
        p.body[b] = bs;
        sh_q = q;
        sh_X[0] = bs.pos.x;
        sh_X[1] = bs.pos.y;
        sh_X[2] = bs.pos.z;
    }
    __syncthreads();

    // ---- 3. the members follow ----
    const Quat q = sh_q, qi = qinverse(sh_q);
    int pend = 0;
    for (int m = m0 + threadIdx.x; m < m1; m += blockDim.x)
    {
        const int s = p.inv[p.body_ids[m]];
        const float4 p0 = p.body_p0[m];
        const Quat r = qmul(qmul(q, Quat{p0.x, p0.y, p0.z, 0.0f}), qi);
        const float4 old = p.pos[sold][s];
        const float nx = __fadd_rn(sh_X[0], r.x), ny = __fadd_rn(sh_X[1], r.y), nz = __fadd_rn(sh_X[2], r.z);
        p.pos[snew][s] = make_float4(nx, ny, nz, old.w);
        p.vel[snew][s] = make_float4(__fdiv_rn(__fsub_rn(nx, old.x), p.dt), __fdiv_rn(__fsub_rn(ny, old.y), p.dt),
                                     __fdiv_rn(__fsub_rn(nz, old.z), p.dt), 0.f);
        if (p.pos_lo[0])
            p.pos_lo[snew][s] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!isfinite(nx) || !isfinite(ny) || !isfinite(nz))
            pend |= ST_NONFINITE;
        const float4 bp = p.pos_build[s];
        const float ddx = nx - bp.x, ddy = ny - bp.y, ddz = nz - bp.z;
        if (ddx * ddx + ddy * ddy + ddz * ddz > p.half_skin2)
            pend |= ST_STALE;
    }
    // raised bits stop the next kernels
    if (pend)
        atomicOr(&ctl->status, pend);
    // the last block records the step as done: every block has passed its check by then
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0)
    {
        __threadfence();
        last = atomicAdd(&ctl->done_rigid, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0)
    {
        ctl->rigid_steps = steps;
        ctl->done_rigid = 0u;
    }
}

} // namespace

int launch_rigid(const Params &p, cudaStream_t st)
{
    k_rigid<<<p.nbody, kRigidBlock, 0, st>>>(p);
    return 1;
}

} // namespace bsg
