// Pose algebra on the device: the exact chain from per-view twist gradients to the
// reference's 12 optimised deltas, the Adam step and the pose / velocity update of the
// batched tracker, and the drop-in helpers (view entry from settings tensors, chain of
// one view's gradient).  The per-view gradient sums are formed from per-block float
// pairs with error-free FP32 arithmetic (about 48 significant bits); the chain, Adam and
// exponential maps run in FP32, as the reference's own pose parameters do, and the pose
// itself is stored and composed in FP64.
//
// Pose conventions follow the reference:
//   SE3_exp([rho, theta]) with the SO(3) left Jacobian V (utils/pose.py:26-91);
//   rendered pair poses T_s = SE3_exp(s [v, w] dtau/2) T, s = -1 / +1
//   (utils/render_camera/camera.py:100-123, frame.py:68-73);
//   update_pose: T <- SE3_exp([rho, theta]) T, deltas reset to 0 (camera.py:133-147);
//   update_vwRT: velocity += (dv, dw) then update_pose (camera.py:129-155);
//   Adam with the four parameter groups theta, rho, w, v (utils/tracker.py:117-129),
//   torch's default betas (0.9, 0.999) and eps 1e-8, groups without a gradient skipped.
// Gradient chain, with g_s = dL/d(left twist of view s):
//   d/d(rho, theta) = sum_s Ad(E_s)^T g_s,
//   d/d(v, w)       = sum_s s h J_l(s h u)^T g_s,  u = [v, w], h = dtau / 2,
// J_l being the exact SE(3) left Jacobian (Barfoot & Furgale, IEEE T-RO 2014).
#include "common.cuh"

namespace {

// 3x3 matrices in FP32: transcendental and divide-heavy math stays off the (slow) FP64
// units; the per-view gradient sums arrive in FP64 and the pose is stored in FP64.
struct M3 { float a[9]; };

__device__ inline M3 m3_eye() { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = (i % 4 == 0) ? 1.0f : 0.0f; return r; }
__device__ inline M3 m3_mul(const M3 &x, const M3 &y)
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r.a[3 * i + j] = x.a[3 * i] * y.a[j] + x.a[3 * i + 1] * y.a[3 + j] + x.a[3 * i + 2] * y.a[6 + j];
    return r;
}
__device__ inline M3 m3_add(const M3 &x, const M3 &y, float sy) { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = x.a[i] + sy * y.a[i]; return r; }
__device__ inline M3 m3_scale(const M3 &x, float s) { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = s * x.a[i]; return r; }
__device__ inline M3 skew(const float *v)
{
    M3 r;
    r.a[0] = 0; r.a[1] = -v[2]; r.a[2] = v[1];
    r.a[3] = v[2]; r.a[4] = 0; r.a[5] = -v[0];
    r.a[6] = -v[1]; r.a[7] = v[0]; r.a[8] = 0;
    return r;
}
__device__ inline void m3_vec(const M3 &m, const float *v, float *o)
{
    for (int i = 0; i < 3; ++i) o[i] = m.a[3 * i] * v[0] + m.a[3 * i + 1] * v[1] + m.a[3 * i + 2] * v[2];
}
__device__ inline void m3t_vec(const M3 &m, const float *v, float *o)
{
    for (int i = 0; i < 3; ++i) o[i] = m.a[i] * v[0] + m.a[3 + i] * v[1] + m.a[6 + i] * v[2];
}

// SO(3) coefficients sin(a)/a, (1-cos a)/a^2, (a - sin a)/a^3 with Taylor series below
// 0.1 rad, where the closed forms lose accuracy in FP32 through cancellation.
__device__ inline void so3_coeffs(float a, float &A, float &B, float &Cc)
{
    float a2 = a * a;
    if (a < 0.1f) {
        A = 1.0f - a2 * (1.0f / 6.0f) + a2 * a2 * (1.0f / 120.0f);
        B = 0.5f - a2 * (1.0f / 24.0f) + a2 * a2 * (1.0f / 720.0f);
        Cc = (1.0f / 6.0f) - a2 * (1.0f / 120.0f) + a2 * a2 * (1.0f / 5040.0f);
    } else {
        float s = sinf(a), c = cosf(a);
        A = s / a;
        B = (1.0f - c) / a2;
        Cc = (a - s) / (a2 * a);
    }
}

__device__ inline M3 so3_exp(const float *th)
{
    M3 W = skew(th), W2 = m3_mul(W, W);
    float A, B, Cc;
    so3_coeffs(sqrtf(th[0] * th[0] + th[1] * th[1] + th[2] * th[2]), A, B, Cc);
    return m3_add(m3_add(m3_eye(), W, A), W2, B);
}

// SO(3) left Jacobian V(theta) (utils/pose.py:61-76)
__device__ inline M3 so3_jl(const float *th)
{
    M3 W = skew(th), W2 = m3_mul(W, W);
    float A, B, Cc;
    so3_coeffs(sqrtf(th[0] * th[0] + th[1] * th[1] + th[2] * th[2]), A, B, Cc);
    return m3_add(m3_add(m3_eye(), W, B), W2, Cc);
}

// SE3_exp(xi = [rho, theta]) -> R, t
__device__ inline void se3_exp(const float *xi, M3 &R, float *t)
{
    R = so3_exp(xi + 3);
    M3 V = so3_jl(xi + 3);
    m3_vec(V, xi, t);
}

// Q block of the SE(3) left Jacobian
__device__ inline M3 se3_q(const float *xi)
{
    const float *rho = xi, *phi = xi + 3;
    M3 P = skew(phi), Rh = skew(rho);
    M3 PR = m3_mul(P, Rh), RP = m3_mul(Rh, P), PRP = m3_mul(PR, P);
    M3 PPR = m3_mul(P, PR), RPP = m3_mul(RP, P);
    M3 PRPP = m3_mul(PRP, P), PPRP = m3_mul(P, PRP);
    float a = sqrtf(phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2]);
    float a2 = a * a;
    float c1, c2, c3;
    if (a < 0.1f) {
        c1 = (1.0f / 6.0f) - a2 * (1.0f / 120.0f) + a2 * a2 * (1.0f / 5040.0f);
        c2 = (1.0f / 24.0f) - a2 * (1.0f / 720.0f) + a2 * a2 * (1.0f / 40320.0f);
        c3 = (1.0f / 120.0f) - a2 * (1.0f / 2520.0f) + a2 * a2 * (1.0f / 120960.0f);
    } else {
        float s = sinf(a), c = cosf(a), a3 = a2 * a, a4 = a3 * a, a5 = a4 * a;
        c1 = (a - s) / a3;
        c2 = (a2 + 2.0f * c - 2.0f) / (2.0f * a4);
        c3 = (2.0f * a - 3.0f * s + a * c) / (2.0f * a5);
    }
    M3 A = m3_add(m3_add(PR, RP, 1.0f), PRP, 1.0f);
    M3 B = m3_add(m3_add(PPR, RPP, 1.0f), PRP, -3.0f);
    M3 C = m3_add(PRPP, PPRP, 1.0f);
    M3 Q = m3_scale(Rh, 0.5f);
    Q = m3_add(Q, A, c1);
    Q = m3_add(Q, B, c2);
    Q = m3_add(Q, C, c3);
    return Q;
}

// out6 += Ad(E)^T g  with E = (R, t): Ad = [[R, [t]x R], [0, R]]  (twists [rho, theta])
__device__ inline void adjoint_t_acc(const M3 &R, const float *t, const float *g, float *out6)
{
    float a[3], b[3], c[3];
    m3t_vec(R, g, a);
    M3 txR = m3_mul(skew(t), R);
    m3t_vec(txR, g, b);
    m3t_vec(R, g + 3, c);
    for (int i = 0; i < 3; ++i) { out6[i] += a[i]; out6[3 + i] += b[i] + c[i]; }
}

// out6 += sc * J_l(xi)^T g,  J_l = [[J, Q], [0, J]]
__device__ inline void jl_t_acc(const float *xi, const float *g, float sc, float *out6)
{
    M3 J = so3_jl(xi + 3), Q = se3_q(xi);
    float a[3], b[3], c[3];
    m3t_vec(J, g, a);
    m3t_vec(Q, g, b);
    m3t_vec(J, g + 3, c);
    for (int i = 0; i < 3; ++i) { out6[i] += sc * a[i]; out6[3 + i] += sc * (b[i] + c[i]); }
}


// rendered pose of role s (-1 last, +1 next): E_s T, with E_s = SE3_exp(s h [v, w]); the
// view entries are FP32, so the product is formed in FP32 from the rounded pose.
__device__ inline void pair_pose(const gsevt_pose_state &S, float sgn, float *Rs, float *ts, M3 &RE, float *tE)
{
    float h = (float)(S.delta_tau * 0.5);
    float u[6] = {sgn * h * (float)S.lin_vel[0], sgn * h * (float)S.lin_vel[1], sgn * h * (float)S.lin_vel[2],
                  sgn * h * (float)S.ang_vel[0], sgn * h * (float)S.ang_vel[1], sgn * h * (float)S.ang_vel[2]};
    se3_exp(u, RE, tE);
    float R[9], t[3];
    for (int i = 0; i < 9; ++i) R[i] = (float)S.R[i];
    for (int i = 0; i < 3; ++i) t[i] = (float)S.t[i];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            Rs[3 * i + j] = RE.a[3 * i] * R[j] + RE.a[3 * i + 1] * R[3 + j] + RE.a[3 * i + 2] * R[6 + j];
        ts[i] = ((RE.a[3 * i] * t[0] + RE.a[3 * i + 1] * t[1]) + RE.a[3 * i + 2] * t[2]) + tE[i];
    }
}

__device__ inline void write_view_pose(gsevt_view *V, const float *R, const float *t)
{
    for (int i = 0; i < 9; ++i) V->R[i] = R[i];
    for (int i = 0; i < 3; ++i) V->t[i] = t[i];
    for (int i = 0; i < 3; ++i) V->campos[i] = -(R[i] * t[0] + R[3 + i] * t[1] + R[6 + i] * t[2]);
}

// One block per pose.  The block sums the per-scan-block twist partials of the pose's two
// views as float pairs with error-free FP32 transformations (about 48 significant bits;
// GB300's FP64 rate would make plain double sums the slowest part of the kernel): each
// view by half of the block, thread i adding partials i, i + 128, ... in order, four loads
// in flight, then warp and block combinations in a fixed order.  The pose state is staged in shared memory.  Warp 0 then runs the serial part with its lanes sharing the
// independent pieces: the two views' chain terms (lanes 0, 1), the four Adam groups
// (lanes 0-3), the pose update (lane 0) and the two view rewrites (lanes 0, 1).
// threads of the finalize block: half of them reduce each view's twist partials
#define FIN_THREADS 512
__global__ void __launch_bounds__(FIN_THREADS) k_track_finalize(gsevt_view *views, const gsevt_map *maps,
                                                             gsevt_pose_state *poses, int num_poses, Workspace ws,
                                                             const double *loss, gsevt_pair *pairs, int num_pairs)
{
    __shared__ float2 part[2][FIN_THREADS / 32][6];
    __shared__ gsevt_pose_state S;
    __shared__ float s_g[2][6], s_acc[2][12], s_grad[12], s_delta[12];
    __shared__ int s_ok;
    constexpr int WORDS = (int)(sizeof(gsevt_pose_state) / 4);
    const int pi = blockIdx.x;
    if (pi >= num_poses) return;
    // the iteration's sort gave up: leave the pose state as it is (uniform)
    if (gs_sort_timed_out(ws.status)) return;
    if (poses[pi].control && poses[pi].frozen) return;  // this problem's level is finished (uniform)
    for (int i = threadIdx.x; i < WORDS; i += FIN_THREADS)
        ((uint32_t *)&S)[i] = ((const uint32_t *)(poses + pi))[i];
    __syncthreads();
    const int vids[2] = {S.last_view, S.next_view};
    {
        // the two views are reduced concurrently, each by half of the block
        constexpr int HALF = FIN_THREADS / 2;
        const int k = threadIdx.x / HALF, t = threadIdx.x % HALF;
        const gsevt_view &V = views[vids[k]];
        const int nb = (maps[V.map].n + GS_BLOCK - 1) / GS_BLOCK;
        const float2 *xp = (const float2 *)ws.xi_part + (size_t)V.sb_offset * 6;
        FP2 acc[6];
        for (int i0 = t; i0 < nb; i0 += 4 * HALF) {
            float2 x[4][6];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = i0 + j * HALF;
#pragma unroll
                for (int q = 0; q < 6; ++q) x[j][q] = i < nb ? xp[(size_t)i * 6 + q] : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int q = 0; q < 6; ++q) acc[q].add(x[j][q].x, x[j][q].y);
        }
        for (int q = 0; q < 6; ++q) {
            FP2 sm = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float hi = __shfl_xor_sync(0xffffffffu, sm.hi, o), lo = __shfl_xor_sync(0xffffffffu, sm.lo, o);
                // combine in lane order so that both partners form the same sum
                FP2 oth;
                oth.hi = hi;
                oth.lo = lo;
                FP2 a = ((threadIdx.x & o) == 0) ? sm : oth;
                const FP2 b2 = ((threadIdx.x & o) == 0) ? oth : sm;
                a.add(b2.hi, b2.lo);
                sm = a;
            }
            if ((t & 31) == 0) part[k][t >> 5][q] = make_float2(sm.hi, sm.lo);
        }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x / 6, q = threadIdx.x % 6;
        FP2 sm;
        for (int w = 0; w < FIN_THREADS / 64; ++w) sm.add(part[k][w][q].x, part[k][w][q].y);
        const double v = (double)sm.hi + (double)sm.lo;
        ws.xi[6 * vids[k] + q] = v;
        s_g[k][q] = (float)v;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    const float h = (float)(S.delta_tau * 0.5);
    const float sg[2] = {-1.0f, 1.0f};
    // chain of each view's twist gradient (lane k: view k)
    if (lane < 2) {
        const int k = lane;
        float g[6];
        for (int i = 0; i < 6; ++i) g[i] = s_g[k][i];
        float u[6] = {sg[k] * h * (float)S.lin_vel[0], sg[k] * h * (float)S.lin_vel[1], sg[k] * h * (float)S.lin_vel[2],
                      sg[k] * h * (float)S.ang_vel[0], sg[k] * h * (float)S.ang_vel[1], sg[k] * h * (float)S.ang_vel[2]};
        float gp[6] = {0, 0, 0, 0, 0, 0}, gv[6] = {0, 0, 0, 0, 0, 0};
        M3 RE;
        float tE[3];
        se3_exp(u, RE, tE);
        adjoint_t_acc(RE, tE, g, gp);
        jl_t_acc(u, g, sg[k] * h, gv);
        for (int i = 0; i < 6; ++i) { s_acc[k][i] = gp[i]; s_acc[k][6 + i] = gv[i]; }
    }
    __syncwarp();
    if (lane == 0) {
        float gpose[6], gvel[6];
        for (int i = 0; i < 6; ++i) {
            gpose[i] = s_acc[0][i] + s_acc[1][i];
            gvel[i] = s_acc[0][6 + i] + s_acc[1][6 + i];
        }
        // 12-vector in the reference's group order: theta, rho, w, v
        float grad[12];
        for (int i = 0; i < 3; ++i) {
            grad[i] = gpose[3 + i];
            grad[3 + i] = gpose[i];
            grad[6 + i] = gvel[3 + i];
            grad[9 + i] = gvel[i];
        }
        bool finite = true;
        for (int i = 0; i < 12; ++i) {
            S.grad[i] = (double)grad[i];
            s_grad[i] = grad[i];
            finite &= isfinite(grad[i]);
        }
        for (int p = 0; p < num_pairs; ++p)
            if (pairs[p].pose == pi) S.loss = loss ? loss[p] : ws.loss_scal[p].L;
        s_ok = finite;
        if (!finite) atomicOr(ws.status, GSEVT_STATUS_NONFINITE);
        // stage control: the velocity learning-rate ramp of the fine stage
        // (utils/tracker.py:188-202): k = optim_iter - start_vel_opt_iter,
        // fraction = k / (max_optim_iter / 2) for 1 <= k <= max_optim_iter / 2, else 1;
        // theta, rho use lr * fraction and w, v use lr * (1 - fraction).
        if (finite && S.control) {
            if (S.opt_vel) {
                const double fnum = 0.5 * (double)S.max_iter;
                const int k = S.level_iter - S.start_vel;
                const double frac = (k >= 1 && (double)k <= fnum) ? (double)k / fnum : 1.0;
                S.lr_scale[0] = S.lr_scale[1] = frac;
                S.lr_scale[2] = S.lr_scale[3] = 1.0 - frac;
            } else {
                S.lr_scale[0] = S.lr_scale[1] = S.lr_scale[2] = S.lr_scale[3] = 1.0;
            }
        }
    }
    __syncwarp();
    if (s_ok) {
        // Adam with torch's update rule, one parameter group per lane; the parameter is 0
        // before every step (the deltas are reset after each update), so the new delta is
        // the step itself
        if (lane < 4) {
            const int gi = lane;
            const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
            const bool active = gi < 2 || S.opt_vel;
            for (int k = 0; k < 3; ++k) s_delta[3 * gi + k] = 0.0f;
            if (active) {
                S.step[gi] += 1;
                const float bc1 = 1.0f - powf(b1, (float)S.step[gi]);
                const float bc2 = 1.0f - powf(b2, (float)S.step[gi]);
                const float lr = (float)(S.lr[gi] * S.lr_scale[gi]);
                for (int k = 0; k < 3; ++k) {
                    const int i = 3 * gi + k;
                    const float gr = s_grad[i];
                    const float m = b1 * (float)S.m[i] + (1.0f - b1) * gr;
                    const float v = b2 * (float)S.v[i] + (1.0f - b2) * gr * gr;
                    S.m[i] = m;
                    S.v[i] = v;
                    const float denom = sqrtf(v) / sqrtf(bc2) + eps;
                    s_delta[i] = -(lr / bc1) * m / denom;
                }
            }
        }
        __syncwarp();
        {
            // update_pose: T <- SE3_exp([rho, theta]) T, the FP64 product spread over lanes
            // 0-11 (one entry each; every lane forms the same FP32 exponential)
            float xi[6] = {s_delta[3], s_delta[4], s_delta[5], s_delta[0], s_delta[1], s_delta[2]};
            M3 Rd;
            float td[3];
            se3_exp(xi, Rd, td);
            double nv = 0.0;
            if (lane < 9) {
                const int i = lane / 3, j = lane % 3;
                nv = (double)Rd.a[3 * i] * S.R[j] + (double)Rd.a[3 * i + 1] * S.R[3 + j] +
                     (double)Rd.a[3 * i + 2] * S.R[6 + j];
            } else if (lane < 12) {
                const int i = lane - 9;
                nv = (double)Rd.a[3 * i] * S.t[0] + (double)Rd.a[3 * i + 1] * S.t[1] +
                     (double)Rd.a[3 * i + 2] * S.t[2] + (double)td[i];
            }
            __syncwarp();
            if (lane < 9) S.R[lane] = nv;
            else if (lane < 12) S.t[lane - 9] = nv;
            __syncwarp();
        }
        if (lane == 0) {
            // update_vwRT: velocity first (the pose update above uses only the deltas)
            if (S.opt_vel)
                for (int k = 0; k < 3; ++k) { S.ang_vel[k] += s_delta[6 + k]; S.lin_vel[k] += s_delta[9 + k]; }
            S.iter += 1;
            if (S.control) {
                // losses.append(loss); converged = mean |diff(last 11 losses)| < threshold
                // (utils/tracker.py:65-76, 213-217); stage switch / level end (:224-240)
                S.hist[S.hist_n % 11] = S.loss;
                S.hist_n += 1;
                bool converged = false;
                if (S.hist_n > 10) {
                    double acc = 0.0;
                    for (int q = 0; q < 10; ++q) {
                        const double a = S.hist[(S.hist_n - 11 + q) % 11], b = S.hist[(S.hist_n - 10 + q) % 11];
                        acc += fabs(b - a);
                    }
                    converged = acc / 10.0 < S.conv_thr;
                }
                if (converged) {
                    if (!S.opt_vel) {
                        S.opt_vel = 1;
                        S.start_vel = S.level_iter;
                        for (int p = 0; p < num_pairs; ++p)
                            if (pairs[p].pose == pi) pairs[p].unsigned_mode = 0;
                    } else {
                        S.frozen = 1;
                    }
                }
                if (!S.frozen) {
                    if (!S.opt_vel ? (S.level_iter >= S.max_iter) : (S.level_iter >= S.start_vel + S.max_iter))
                        S.frozen = 1;
                }
                S.level_iter += 1;
            }
        }
        __syncwarp();
        // rewrite the pair's view entries for the next iteration (lane k: view k)
        if (lane < 2) {
            float Rs[9], ts[3];
            M3 RE;
            float tE[3];
            pair_pose(S, sg[lane], Rs, ts, RE, tE);
            write_view_pose(views + vids[lane], Rs, ts);
            // a problem whose level just finished renders nothing until the host resets it
            views[vids[lane]].skip = (S.control && S.frozen) ? 1 : 0;
        }
    }
    __syncwarp();
    for (int i = lane; i < WORDS; i += 32) ((uint32_t *)(poses + pi))[i] = ((const uint32_t *)&S)[i];
}

// Initialise the two view entries of every pose from its current state.
__global__ void k_track_views(gsevt_view *views, const gsevt_pose_state *poses, int num_poses)
{
    int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= num_poses) return;
    const gsevt_pose_state &S = poses[pi];
    const int vids[2] = {S.last_view, S.next_view};
    const float sg[2] = {-1.0f, 1.0f};
    for (int k = 0; k < 2; ++k) {
        float Rs[9], ts[3];
        M3 RE;
        float tE[3];
        pair_pose(S, sg[k], Rs, ts, RE, tE);
        write_view_pose(views + vids[k], Rs, ts);
        views[vids[k]].skip = (S.control && S.frozen) ? 1 : 0;
    }
}

__global__ void k_chain_view(const double *xi, const float *E_t, float dt, const float *lin, const float *ang,
                             float *out12)
{
    M3 R;
    float t[3], g[6];
    // E_t is the transposed 4x4 (row-major storage of E^T): E[i][j] = E_t[4 j + i]
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R.a[3 * i + j] = E_t[4 * j + i];
    for (int i = 0; i < 3; ++i) t[i] = E_t[12 + i];
    for (int i = 0; i < 6; ++i) g[i] = (float)xi[i];
    float gpose[6] = {0, 0, 0, 0, 0, 0}, gvel[6] = {0, 0, 0, 0, 0, 0};
    adjoint_t_acc(R, t, g, gpose);
    float u[6] = {dt * lin[0], dt * lin[1], dt * lin[2], dt * ang[0], dt * ang[1], dt * ang[2]};
    if (dt != 0.0f) jl_t_acc(u, g, dt, gvel);
    for (int i = 0; i < 3; ++i) {
        out12[i] = gpose[3 + i];
        out12[3 + i] = gpose[i];
        out12[6 + i] = gvel[3 + i];
        out12[9 + i] = gvel[i];
    }
}

__global__ void k_view_from_settings(const float *vm_t, const float *pr_t, const float *campos, const float *bg,
                                     float tanfx, float tanfy, int W, int H, int tile_offset, int pix_offset,
                                     int map, int vg_offset, int sb_offset, gsevt_view *out)
{
    gsevt_view V;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V.R[3 * i + j] = vm_t[4 * j + i];
    for (int i = 0; i < 3; ++i) V.t[i] = vm_t[12 + i];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) V.P[4 * i + j] = pr_t[4 * j + i];
    for (int i = 0; i < 3; ++i) V.campos[i] = campos[i];
    V.tanfovx = tanfx;
    V.tanfovy = tanfy;
    for (int i = 0; i < 3; ++i) V.bg[i] = bg ? bg[i] : 0.0f;
    V.width = W;
    V.height = H;
    V.tiles_x = (W + GSEVT_TILE - 1) / GSEVT_TILE;
    V.tiles_y = (H + GSEVT_TILE - 1) / GSEVT_TILE;
    V.tile_offset = tile_offset;
    V.pix_offset = pix_offset;
    V.map = map;
    V.vg_offset = vg_offset;
    V.sb_offset = sb_offset;
    V.pair = -1;
    V.pair_role = 0;
    V.skip = 0;
    *out = V;
}

}  // namespace

int gs_launch_track_finalize(const gsevt_frame *f, const Workspace &ws, gsevt_pose_state *poses, int num_poses,
                             const double *loss, cudaStream_t s)
{
    k_track_finalize<<<num_poses, FIN_THREADS, 0, s>>>((gsevt_view *)f->views, f->maps, poses, num_poses, ws, loss,
                                                    (gsevt_pair *)f->pairs, f->L.num_pairs);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_track_init_views(gsevt_view *views, const gsevt_pose_state *poses, int32_t num_poses,
                                      gsevt_stream_t stream)
{
    GS_ENTRY();
    if (!views || !poses || num_poses <= 0) return GSEVT_ERR_ARG;
    k_track_views<<<(num_poses + 63) / 64, 64, 0, (cudaStream_t)stream>>>(views, poses, num_poses);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_chain_view_grad(const double *xi, const float *vel_transform_t, float delta_time,
                                     const float *linear_vel, const float *angular_vel, float *out12,
                                     gsevt_stream_t stream)
{
    GS_ENTRY();
    if (!xi || !vel_transform_t || !linear_vel || !angular_vel || !out12) return GSEVT_ERR_ARG;
    k_chain_view<<<1, 1, 0, (cudaStream_t)stream>>>(xi, vel_transform_t, delta_time, linear_vel, angular_vel, out12);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_view_from_settings(const float *viewmatrix_t, const float *projmatrix_raw_t, const float *campos,
                                        const float *bg, float tanfovx, float tanfovy, int32_t width, int32_t height,
                                        int32_t tile_offset, int32_t pix_offset, int32_t map, int32_t vg_offset,
                                        int32_t sb_offset, gsevt_view *view_out, gsevt_stream_t stream)
{
    GS_ENTRY();
    if (!viewmatrix_t || !projmatrix_raw_t || !campos || !view_out || width <= 0 || height <= 0) return GSEVT_ERR_ARG;
    k_view_from_settings<<<1, 1, 0, (cudaStream_t)stream>>>(viewmatrix_t, projmatrix_raw_t, campos, bg, tanfovx, tanfovy,
                                                           width, height, tile_offset, pix_offset, map, vg_offset,
                                                           sb_offset, view_out);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
