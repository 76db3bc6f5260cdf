// FP64 pose algebra on the device: the exact chain from per-view twist gradients to the
// reference's 12 optimised deltas, the Adam step and the pose / velocity update of the
// batched tracker, and the drop-in helpers (view entry from settings tensors, chain of
// one view's gradient).
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

struct M3 { double a[9]; };

__device__ inline M3 m3_eye() { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = (i % 4 == 0) ? 1.0 : 0.0; return r; }
__device__ inline M3 m3_mul(const M3 &x, const M3 &y)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.a[3 * i + j] = x.a[3 * i] * y.a[j] + x.a[3 * i + 1] * y.a[3 + j] + x.a[3 * i + 2] * y.a[6 + j];
    return r;
}
__device__ inline M3 m3_add(const M3 &x, const M3 &y, double sy) { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = x.a[i] + sy * y.a[i]; return r; }
__device__ inline M3 m3_scale(const M3 &x, double s) { M3 r; for (int i = 0; i < 9; ++i) r.a[i] = s * x.a[i]; return r; }
__device__ inline M3 skew(const double *v)
{
    M3 r;
    r.a[0] = 0; r.a[1] = -v[2]; r.a[2] = v[1];
    r.a[3] = v[2]; r.a[4] = 0; r.a[5] = -v[0];
    r.a[6] = -v[1]; r.a[7] = v[0]; r.a[8] = 0;
    return r;
}
__device__ inline void m3_vec(const M3 &m, const double *v, double *o)
{
    for (int i = 0; i < 3; ++i) o[i] = m.a[3 * i] * v[0] + m.a[3 * i + 1] * v[1] + m.a[3 * i + 2] * v[2];
}
__device__ inline void m3t_vec(const M3 &m, const double *v, double *o)
{
    for (int i = 0; i < 3; ++i) o[i] = m.a[i] * v[0] + m.a[3 + i] * v[1] + m.a[6 + i] * v[2];
}

// SO3_exp with the reference's small-angle branch (utils/pose.py:26-41)
__device__ inline M3 so3_exp(const double *th)
{
    M3 W = skew(th), W2 = m3_mul(W, W);
    double a = sqrt(th[0] * th[0] + th[1] * th[1] + th[2] * th[2]);
    if (a < 1e-5) return m3_add(m3_add(m3_eye(), W, 1.0), W2, 0.5);
    return m3_add(m3_add(m3_eye(), W, sin(a) / a), W2, (1.0 - cos(a)) / (a * a));
}

// V(theta) (utils/pose.py:61-76)
__device__ inline M3 so3_jl(const double *th)
{
    M3 W = skew(th), W2 = m3_mul(W, W);
    double a = sqrt(th[0] * th[0] + th[1] * th[1] + th[2] * th[2]);
    if (a < 1e-5) return m3_add(m3_add(m3_eye(), W, 0.5), W2, 1.0 / 6.0);
    return m3_add(m3_add(m3_eye(), W, (1.0 - cos(a)) / (a * a)), W2, (a - sin(a)) / (a * a * a));
}

// SE3_exp(xi = [rho, theta]) -> R, t
__device__ inline void se3_exp(const double *xi, M3 &R, double *t)
{
    R = so3_exp(xi + 3);
    M3 V = so3_jl(xi + 3);
    m3_vec(V, xi, t);
}

// Q block of the SE(3) left Jacobian
__device__ inline M3 se3_q(const double *xi)
{
    const double *rho = xi, *phi = xi + 3;
    M3 P = skew(phi), Rh = skew(rho);
    M3 PR = m3_mul(P, Rh), RP = m3_mul(Rh, P), PRP = m3_mul(PR, P);
    M3 PPR = m3_mul(P, PR), RPP = m3_mul(RP, P);
    M3 PRPP = m3_mul(PRP, P), PPRP = m3_mul(P, PRP);
    double a = sqrt(phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2]);
    double c1, c2, c3;
    if (a < 1e-4) {
        c1 = 1.0 / 6.0; c2 = 1.0 / 24.0; c3 = 1.0 / 120.0;
    } else {
        double a2 = a * a, a3 = a2 * a, a4 = a3 * a, a5 = a4 * a;
        c1 = (a - sin(a)) / a3;
        c2 = (a2 + 2.0 * cos(a) - 2.0) / (2.0 * a4);
        c3 = (2.0 * a - 3.0 * sin(a) + a * cos(a)) / (2.0 * a5);
    }
    M3 A = m3_add(m3_add(PR, RP, 1.0), PRP, 1.0);
    M3 B = m3_add(m3_add(PPR, RPP, 1.0), PRP, -3.0);
    M3 C = m3_add(PRPP, PPRP, 1.0);
    M3 Q = m3_scale(Rh, 0.5);
    Q = m3_add(Q, A, c1);
    Q = m3_add(Q, B, c2);
    Q = m3_add(Q, C, c3);
    return Q;
}

// out6 += Ad(E)^T g  with E = (R, t): Ad = [[R, [t]x R], [0, R]]  (twists [rho, theta])
__device__ inline void adjoint_t_acc(const M3 &R, const double *t, const double *g, double *out6)
{
    double a[3], b[3], c[3];
    m3t_vec(R, g, a);                 // R^T g_rho
    M3 tx = skew(t);
    M3 txR = m3_mul(tx, R);
    m3t_vec(txR, g, b);               // ([t]x R)^T g_rho
    m3t_vec(R, g + 3, c);             // R^T g_theta
    for (int i = 0; i < 3; ++i) { out6[i] += a[i]; out6[3 + i] += b[i] + c[i]; }
}

// out6 += sc * J_l(xi)^T g,  J_l = [[J, Q], [0, J]]
__device__ inline void jl_t_acc(const double *xi, const double *g, double sc, double *out6)
{
    M3 J = so3_jl(xi + 3), Q = se3_q(xi);
    double a[3], b[3], c[3];
    m3t_vec(J, g, a);
    m3t_vec(Q, g, b);
    m3t_vec(J, g + 3, c);
    for (int i = 0; i < 3; ++i) { out6[i] += sc * a[i]; out6[3 + i] += sc * (b[i] + c[i]); }
}

__device__ inline void write_view_pose(gsevt_view *V, const M3 &R, const double *t)
{
    for (int i = 0; i < 9; ++i) V->R[i] = (float)R.a[i];
    for (int i = 0; i < 3; ++i) V->t[i] = (float)t[i];
    double c[3];
    m3t_vec(R, t, c);
    for (int i = 0; i < 3; ++i) V->campos[i] = (float)(-c[i]);
}

// rendered pose of role s (-1 last, +1 next): E_s T
__device__ inline void pair_pose(const gsevt_pose_state &S, double sgn, M3 &Rs, double *ts, M3 &RE, double *tE)
{
    double h = S.delta_tau * 0.5;
    double u[6] = {sgn * h * S.lin_vel[0], sgn * h * S.lin_vel[1], sgn * h * S.lin_vel[2],
                   sgn * h * S.ang_vel[0], sgn * h * S.ang_vel[1], sgn * h * S.ang_vel[2]};
    se3_exp(u, RE, tE);
    M3 R;
    for (int i = 0; i < 9; ++i) R.a[i] = S.R[i];
    Rs = m3_mul(RE, R);
    double Et[3];
    m3_vec(RE, S.t, Et);
    for (int i = 0; i < 3; ++i) ts[i] = Et[i] + tE[i];
}

__global__ void k_track_finalize(gsevt_view *views, gsevt_pose_state *poses, int num_poses, Workspace ws,
                                 const double *loss, const gsevt_pair *pairs, int num_pairs)
{
    int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= num_poses) return;
    gsevt_pose_state S = poses[pi];
    double h = S.delta_tau * 0.5;
    double gpose[6] = {0, 0, 0, 0, 0, 0}, gvel[6] = {0, 0, 0, 0, 0, 0};
    const int vids[2] = {S.last_view, S.next_view};
    const double sg[2] = {-1.0, 1.0};
    for (int k = 0; k < 2; ++k) {
        const double *g = ws.xi + 6 * vids[k];
        M3 Rs, RE;
        double ts[3], tE[3];
        pair_pose(S, sg[k], Rs, ts, RE, tE);
        adjoint_t_acc(RE, tE, g, gpose);
        double u[6] = {sg[k] * h * S.lin_vel[0], sg[k] * h * S.lin_vel[1], sg[k] * h * S.lin_vel[2],
                       sg[k] * h * S.ang_vel[0], sg[k] * h * S.ang_vel[1], sg[k] * h * S.ang_vel[2]};
        jl_t_acc(u, g, sg[k] * h, gvel);
    }
    // 12-vector in the reference's group order: theta, rho, w, v
    double grad[12];
    for (int i = 0; i < 3; ++i) {
        grad[i] = gpose[3 + i];
        grad[3 + i] = gpose[i];
        grad[6 + i] = gvel[3 + i];
        grad[9 + i] = gvel[i];
    }
    for (int i = 0; i < 12; ++i) S.grad[i] = grad[i];
    for (int p = 0; p < num_pairs; ++p)
        if (pairs[p].pose == pi) S.loss = loss ? loss[p] : ws.loss_scal[4 * p + 3];
    bool finite = true;
    for (int i = 0; i < 12; ++i) finite &= isfinite(grad[i]);
    if (!finite) {
        atomicOr(ws.status, GSEVT_STATUS_NONFINITE);
        poses[pi] = S;
        return;
    }
    // Adam (torch semantics): param starts at 0 every step (deltas are reset after the update)
    double delta[12];
    const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    for (int gi = 0; gi < 4; ++gi) {
        bool active = gi < 2 || S.opt_vel;
        for (int k = 0; k < 3; ++k) delta[3 * gi + k] = 0.0;
        if (!active) continue;
        S.step[gi] += 1;
        double bc1 = 1.0 - pow(b1, (double)S.step[gi]);
        double bc2 = 1.0 - pow(b2, (double)S.step[gi]);
        double lr = S.lr[gi] * S.lr_scale[gi];
        for (int k = 0; k < 3; ++k) {
            int i = 3 * gi + k;
            S.m[i] = b1 * S.m[i] + (1.0 - b1) * grad[i];
            S.v[i] = b2 * S.v[i] + (1.0 - b2) * grad[i] * grad[i];
            double denom = sqrt(S.v[i]) / sqrt(bc2) + eps;
            delta[i] = -(lr / bc1) * S.m[i] / denom;
        }
    }
    // update_vwRT: velocity first, then the pose
    if (S.opt_vel)
        for (int k = 0; k < 3; ++k) { S.ang_vel[k] += delta[6 + k]; S.lin_vel[k] += delta[9 + k]; }
    double xi[6] = {delta[3], delta[4], delta[5], delta[0], delta[1], delta[2]};
    M3 Rd;
    double td[3];
    se3_exp(xi, Rd, td);
    M3 R;
    for (int i = 0; i < 9; ++i) R.a[i] = S.R[i];
    M3 Rn = m3_mul(Rd, R);
    double tn[3];
    m3_vec(Rd, S.t, tn);
    for (int i = 0; i < 3; ++i) tn[i] += td[i];
    for (int i = 0; i < 9; ++i) S.R[i] = Rn.a[i];
    for (int i = 0; i < 3; ++i) S.t[i] = tn[i];
    S.iter += 1;
    // rewrite the pair's view entries for the next iteration
    for (int k = 0; k < 2; ++k) {
        M3 Rs, RE;
        double ts[3], tE[3];
        pair_pose(S, sg[k], Rs, ts, RE, tE);
        write_view_pose(views + vids[k], Rs, ts);
    }
    poses[pi] = S;
}

// Initialise the two view entries of every pose from its current state.
__global__ void k_track_views(gsevt_view *views, const gsevt_pose_state *poses, int num_poses)
{
    int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= num_poses) return;
    gsevt_pose_state S = poses[pi];
    const int vids[2] = {S.last_view, S.next_view};
    const double sg[2] = {-1.0, 1.0};
    for (int k = 0; k < 2; ++k) {
        M3 Rs, RE;
        double ts[3], tE[3];
        pair_pose(S, sg[k], Rs, ts, RE, tE);
        write_view_pose(views + vids[k], Rs, ts);
    }
}

__global__ void k_chain_view(const double *xi, const float *E_t, float dt, const float *lin, const float *ang,
                             float *out12)
{
    M3 R;
    double t[3];
    // E_t is the transposed 4x4 (row-major storage of E^T): E[i][j] = E_t[4 j + i]
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R.a[3 * i + j] = (double)E_t[4 * j + i];
    for (int i = 0; i < 3; ++i) t[i] = (double)E_t[12 + i];
    double gpose[6] = {0, 0, 0, 0, 0, 0}, gvel[6] = {0, 0, 0, 0, 0, 0};
    adjoint_t_acc(R, t, xi, gpose);
    double d = (double)dt;
    double u[6] = {d * lin[0], d * lin[1], d * lin[2], d * ang[0], d * ang[1], d * ang[2]};
    if (d != 0.0) jl_t_acc(u, xi, d, gvel);
    for (int i = 0; i < 3; ++i) {
        out12[i] = (float)gpose[3 + i];
        out12[3 + i] = (float)gpose[i];
        out12[6 + i] = (float)gvel[3 + i];
        out12[9 + i] = (float)gvel[i];
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
    V.pad = 0;
    *out = V;
}

}  // namespace

int gs_launch_track_finalize(const gsevt_frame *f, const Workspace &ws, gsevt_pose_state *poses, int num_poses,
                             const double *loss, cudaStream_t s)
{
    k_track_finalize<<<(num_poses + 63) / 64, 64, 0, s>>>((gsevt_view *)f->views, poses, num_poses, ws, loss,
                                                          f->pairs, f->L.num_pairs);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_track_init_views(gsevt_view *views, const gsevt_pose_state *poses, int32_t num_poses,
                                      gsevt_stream_t stream)
{
    if (!views || !poses || num_poses <= 0) return GSEVT_ERR_ARG;
    k_track_views<<<(num_poses + 63) / 64, 64, 0, (cudaStream_t)stream>>>(views, poses, num_poses);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}

extern "C" int gsevt_chain_view_grad(const double *xi, const float *vel_transform_t, float delta_time,
                                     const float *linear_vel, const float *angular_vel, float *out12,
                                     gsevt_stream_t stream)
{
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
    if (!viewmatrix_t || !projmatrix_raw_t || !campos || !view_out || width <= 0 || height <= 0) return GSEVT_ERR_ARG;
    k_view_from_settings<<<1, 1, 0, (cudaStream_t)stream>>>(viewmatrix_t, projmatrix_raw_t, campos, bg, tanfovx, tanfovy,
                                                           width, height, tile_offset, pix_offset, map, vg_offset,
                                                           sb_offset, view_out);
    GS_CUDA_CHECK();
    return GSEVT_OK;
}
