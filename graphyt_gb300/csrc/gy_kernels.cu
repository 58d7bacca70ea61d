// gy_kernels.cu -- the GB300 kernels of one explicit GIMP MPM step.
//
//   P2G        particle-centric scatter of mass, momentum, internal+external force (and,
//              with several bodies, per-body fields and normals) into the node grid.  The
//              reference gathers per node over a 4x4x4 cell window (Extrapolation.cpp:31-125,
//              166-286); a particle contributes to exactly the nodes of its GIMP support,
//              so scattering over the 3x3x3 stencil sums the same terms.
//   fold       periodic node-layer fold (Grid.cpp:310-795), one launch per axis.
//   solve      nodal momentum update, contact and grid BCs (Grid.cpp:9-245, 862-1094).
//   G2P+update gather of grid velocity/acceleration/strain rate (Extrapolation.cpp:127-163,
//              288-367), particle BCs (TimeIntegration.cpp:177-296), particle update,
//              constitutive + damage, periodic wrap and the new cell key
//              (TimeIntegration.cpp:11-117), fused in one pass over the particles.
#include <atomic>
#include <cstdio>

#include "gy_kernels.cuh"
#include "gy_physics.cuh"

namespace gy {

static std::atomic<long long> g_launches{0};
void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------------------
// P2G

__device__ __forceinline__ void red_add(float *a, float v)
{
    if (v != 0.0f) atomicAdd(a, v);
}

__device__ __forceinline__ void red_add4(float4 *a, float x, float y, float z, float w)
{
    // vector reduction into global memory (sm_90+): one request for four floats
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(x), "f"(y), "f"(z), "f"(w)
                 : "memory");
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_p2g_global(PView P, long long n, NodeBufs nb, StepArgs a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GridGeom &g = a.g;
    const uint32_t info = (uint32_t)P.ii(PF_INFO, i);
    const int key = P.ii(PF_KEY, i);
    int ci, cj, ck;
    decode_key(key, g, ci, cj, ck);
    float Sx[3], Gx[3], Sy[3], Gy[3], Sz[3] = {1.f, 0.f, 0.f}, Gz[3] = {0.f, 0.f, 0.f};
    const float ox = P.f(PF_OX, i), oy = P.f(PF_OY, i);
    gimp_axis(ox, g.lp, Sx, Gx);
    gimp_axis(oy, g.lp, Sy, Gy);
    int nkz = 1;
    if (g.is3d) {
        const float oz = P.f(PF_OZ, i);
        gimp_axis(oz, g.lp, Sz, Gz);
        nkz = (oz < 1.0f - g.lp) ? 2 : 3;
    } else {
        ck = 0;
    }
    const int nix = (ox < 1.0f - g.lp) ? 2 : 3;
    const int njy = (oy < 1.0f - g.lp) ? 2 : 3;
    const float m = P.f(PF_MASS, i);
    const float rho = P.f(PF_RHO, i);
    const float vx = P.f(PF_VX, i), vy = P.f(PF_VY, i), vz = P.f(PF_VZ, i);
    const float Vf = m / rho;  // force volume m/rho (Extrapolation.cpp:221)
    // V * sigma, with the 1/h of the gradient folded in
    const float sc = Vf * g.inv_h;
    const float s0 = P.f(PF_S0, i) * sc, s1 = P.f(PF_S1, i) * sc, s2 = P.f(PF_S2, i) * sc;
    const float s3 = P.f(PF_S3, i) * sc, s4 = P.f(PF_S4, i) * sc, s5 = P.f(PF_S5, i) * sc;
    const float mgx = m * a.sc.gravity[0], mgy = m * a.sc.gravity[1], mgz = m * a.sc.gravity[2];
    const bool rigid = (info & INFO_RIGID) != 0;
    const int obj = info_obj(info);
    const float vol_n = ((info & INFO_INIT_VOL) ? a.sc.init_volume : Vf) * g.inv_h;  // normals use the stored volume
    for (int kk = 0; kk < nkz; kk++)
        for (int jj = 0; jj < njy; jj++) {
            const float syz = Sy[jj] * Sz[kk], gyz = Gy[jj] * Sz[kk], syg = Sy[jj] * Gz[kk];
            for (int ii = 0; ii < nix; ii++) {
                const float w = Sx[ii] * syz;
                const float gx = Gx[ii] * syz, gy = Sx[ii] * gyz, gz = Sx[ii] * syg;
                const long long nd = node_index(ci + ii, cj + jj, ck + kk, g);
                const float wm = w * m;
                const float fx = -(gx * s0 + gy * s3 + gz * s5);
                const float fy = -(gx * s3 + gy * s1 + gz * s4);
                const float fz = -(gx * s5 + gy * s4 + gz * s2);
                red_add4(&nb.acc0[nd], wm, wm * vx, wm * vy, wm * vz);
                red_add4(&nb.acc1[nd], fx + w * mgx, fy + w * mgy, fz + w * mgz, 0.0f);
                if (MULTI) {
                    const int2 b = nb.body[nd];
                    const int slot = (b.x == obj) ? 0 : ((b.y == obj) ? 1 : -1);
                    if (slot >= 0) {
                        red_add4(&nb.bacc0[slot][nd], wm, wm * vx, wm * vy, wm * vz);
                        if (rigid) red_add4(&nb.bacc1[slot][nd], fx, fy, fz, 0.0f);
                        else red_add4(&nb.bacc1[slot][nd], fx + w * mgx, fy + w * mgy, fz + w * mgz, 0.0f);
                        red_add4(&nb.bnrm[slot][nd], gx * vol_n, gy * vol_n, gz * vol_n, 0.0f);
                    }
                }
            }
        }
}

void launch_p2g(const PView &p, long long n, const NodeBufs &nb, const StepArgs &a, int tile, int block, cudaStream_t s)
{
    (void)tile;
    (void)block;
    if (n == 0) return;
    const int B = 256;
    const unsigned grid = (unsigned)((n + B - 1) / B);
    if (a.sc.multi_body) {
        k_p2g_global<true><<<grid, B, 0, s>>>(p, n, nb, a);
        note_launch(1);
    }
    else {
        k_p2g_global<false><<<grid, B, 0, s>>>(p, n, nb, a);
        note_launch(1);
    }
}

// ---------------------------------------------------------------------------------------
// periodic fold, Grid.cpp:310-795: node i and node N-3+i (i < 3) both take their sum, for
// mass, momentum and force of the centre-of-mass field and both body fields.

__device__ __forceinline__ void fold4(float4 *arr, long long p, long long q)
{
    float4 x = arr[p], y = arr[q];
    float4 s = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
    arr[p] = s;
    arr[q] = s;
}

template <bool MULTI>
__global__ void k_fold(NodeBufs nb, GridGeom g, int axis)
{
    // pairs: 3 layers x the plane orthogonal to `axis`
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int d0, d1, l;  // plane extents
    if (axis == 0) { d0 = g.ny; d1 = g.nz; }
    else if (axis == 1) { d0 = g.nx; d1 = g.nz; }
    else { d0 = g.nx; d1 = g.ny; }
    const long long plane = (long long)d0 * d1;
    if (t >= 3 * plane) return;
    l = (int)(t / plane);
    const long long r = t - (long long)l * plane;
    const int a0 = (int)(r % d0), a1 = (int)(r / d0);
    long long p, q;
    if (axis == 0) { p = node_index(l, a0, a1, g); q = node_index(g.nx - 3 + l, a0, a1, g); }
    else if (axis == 1) { p = node_index(a0, l, a1, g); q = node_index(a0, g.ny - 3 + l, a1, g); }
    else { p = node_index(a0, a1, l, g); q = node_index(a0, a1, g.nz - 3 + l, g); }
    fold4(nb.acc0, p, q);
    fold4(nb.acc1, p, q);
    if (MULTI) {
        for (int b = 0; b < 2; b++) {
            fold4(nb.bacc0[b], p, q);
            fold4(nb.bacc1[b], p, q);
        }
    }
}

void launch_fold(const NodeBufs &nb, const StepArgs &a, cudaStream_t s)
{
    const GridGeom &g = a.g;
    const int naxes = g.is3d ? 3 : 2;
    for (int ax = 0; ax < naxes; ax++) {
        long long plane = ax == 0 ? (long long)g.ny * g.nz : ax == 1 ? (long long)g.nx * g.nz : (long long)g.nx * g.ny;
        long long total = 3 * plane;
        unsigned grid = (unsigned)((total + 255) / 256);
        if (a.sc.multi_body) {
            k_fold<true><<<grid, 256, 0, s>>>(nb, g, ax);
            note_launch(1);
        }
        else {
            k_fold<false><<<grid, 256, 0, s>>>(nb, g, ax);
            note_launch(1);
        }
    }
}

// ---------------------------------------------------------------------------------------
// nodal solve (Grid.cpp:9-245) + grid BC phase 2 (Grid.cpp:862-1094)

struct BCApply {
    int type;
    float4 val;
    int fixed;
    // which components are set and to which value
    __device__ __forceinline__ void comps(bool set[3], float v[3]) const
    {
        set[0] = set[1] = set[2] = false;
        switch (type) {
        case BC_GRID_VX: set[0] = true; v[0] = val.x; break;
        case BC_GRID_VY: set[1] = true; v[1] = val.x; break;
        case BC_GRID_VX_VY: set[0] = set[1] = true; v[0] = val.x; v[1] = val.y; break;
        case BC_GRID_VZ: if (fixed) { set[2] = true; v[2] = val.x; } break;
        case BC_GRID_VX_VZ: if (fixed) { set[0] = set[2] = true; v[0] = val.x; v[2] = val.y; } break;
        case BC_GRID_VY_VZ: if (fixed) { set[1] = set[2] = true; v[1] = val.x; v[2] = val.y; } break;
        case BC_GRID_VX_VY_VZ:
            if (fixed) { set[0] = set[1] = set[2] = true; v[0] = val.x; v[1] = val.y; v[2] = val.z; }
            break;
        default: break;
        }
    }
};

__device__ __forceinline__ void body_update(float m, const float4 &p, const float4 &f, float dtn, float v[3], float acc[3])
{
    v[0] = p.y / m; v[1] = p.z / m; v[2] = p.w / m;
    acc[0] = f.x / m; acc[1] = f.y / m; acc[2] = f.z / m;
    v[0] += acc[0] * dtn; v[1] += acc[1] * dtn; v[2] += acc[2] * dtn;
}

// calculateColoumbFrictionContactNormals, Grid.cpp:247-308 (only the contact normal is
// used by the solve; the friction outputs are discarded by the caller)
__device__ __forceinline__ void contact_normal(const float rv[3], const float n[3], float mu, float cn[3])
{
    float om0 = rv[1] * n[2] - rv[2] * n[1];
    float om1 = rv[0] * n[2] - rv[2] * n[0];
    float om2 = rv[0] * n[1] - rv[1] * n[0];
    const float mag = sqrtf(om0 * om0 + om1 * om1 + om2 * om2) + 0.001f;
    om0 /= mag; om1 /= mag; om2 /= mag;
    const float mu0 = mag / (rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2]) + 0.001f;
    const float on0 = om2 * n[1] - om1 * n[2];
    const float on1 = om2 * n[0] - om0 * n[2];
    const float on2 = om1 * n[0] - om0 * n[1];
    if (mu0 < mu) mu = mu0;
    cn[0] = n[0] + on0 * mu;
    cn[1] = n[1] + on1 * mu;
    cn[2] = n[2] + on2 * mu;
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_solve(NodeBufs nb, StepArgs a, int keep)
{
    const long long nd = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= a.g.nn) return;
    const float4 A0 = nb.acc0[nd], A1 = nb.acc1[nd];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    nb.acc0[nd] = z4;
    nb.acc1[nd] = z4;
    const float m = A0.x;
    const float dtn = a.sc.dt_node, dt = a.sc.dt;
    float vc[3] = {0.f, 0.f, 0.f};
    float v1[3] = {0.f, 0.f, 0.f}, a1[3] = {0.f, 0.f, 0.f};
    float v2[3] = {0.f, 0.f, 0.f}, a2[3] = {0.f, 0.f, 0.f};
    float n1[3] = {0.f, 0.f, 0.f};
    const bool active = (m != 0.0f);
    if (!MULTI) {
        if (active) {
            vc[0] = A0.y / m; vc[1] = A0.z / m; vc[2] = A0.w / m;
            body_update(m, A0, A1, dtn, v1, a1);
        }
    } else {
        float4 B0[2], B1[2], BN[2];
        for (int b = 0; b < 2; b++) {
            B0[b] = nb.bacc0[b][nd];
            B1[b] = nb.bacc1[b][nd];
            BN[b] = nb.bnrm[b][nd];
            nb.bacc0[b][nd] = z4;
            nb.bacc1[b][nd] = z4;
            nb.bnrm[b][nd] = z4;
        }
        if (active) {
            vc[0] = A0.y / m; vc[1] = A0.z / m; vc[2] = A0.w / m;
            const float mag1 = sqrtf(BN[0].x * BN[0].x + BN[0].y * BN[0].y + BN[0].z * BN[0].z);
            if (mag1 > 1e-8f) { n1[0] = BN[0].x / mag1; n1[1] = BN[0].y / mag1; n1[2] = BN[0].z / mag1; }
            const float n2[3] = {-n1[0], -n1[1], -n1[2]};  // Grid.cpp:45-47
            const float m1 = B0[0].x, m2 = B0[1].x;
            const int2 body = nb.body[nd];
            const unsigned char hr = nb.has_rigid[nd];
            if (body.y != -1) {
                float ap1 = 0.f, ap2 = 0.f, rv1[3] = {0.f, 0.f, 0.f}, rv2[3] = {0.f, 0.f, 0.f};
                if (m1 != 0.0f) {
                    rv1[0] = B0[0].y / m1 - vc[0]; rv1[1] = B0[0].z / m1 - vc[1]; rv1[2] = B0[0].w / m1 - vc[2];
                    ap1 = rv1[0] * n1[0] + rv1[1] * n1[1] + rv1[2] * n1[2];
                }
                if (m2 != 0.0f) {
                    rv2[0] = B0[1].y / m2 - vc[0]; rv2[1] = B0[1].z / m2 - vc[1]; rv2[2] = B0[1].w / m2 - vc[2];
                    ap2 = rv2[0] * n2[0] + rv2[1] * n2[1] + rv2[2] * n2[2];
                }
                if (ap1 > 0.01f || ap2 > 0.01f) {
                    if (hr & 1) {
                        // body 1 rigid: body 2 takes body 1's velocity (Grid.cpp:78-91)
                        if (m1 != 0.0f) {
                            v1[0] = B0[0].y / m1; v1[1] = B0[0].z / m1; v1[2] = B0[0].w / m1;
                            if (m2 != 0.0f) {
                                v2[0] = B0[1].y / m2 - (B0[1].y - m2 * v1[0]) / m2;
                                v2[1] = B0[1].z / m2 - (B0[1].z - m2 * v1[1]) / m2;
                                v2[2] = B0[1].w / m2 - (B0[1].w - m2 * v1[2]) / m2;
                            }
                        }
                    } else if (hr & 2) {
                        if (m2 != 0.0f) {
                            v2[0] = B0[1].y / m2; v2[1] = B0[1].z / m2; v2[2] = B0[1].w / m2;
                            if (m1 != 0.0f) {
                                v1[0] = B0[0].y / m1 - (B0[0].y - m1 * v2[0]) / m1;
                                v1[1] = B0[0].z / m1 - (B0[0].z - m1 * v2[1]) / m1;
                                v1[2] = B0[0].w / m1 - (B0[0].w - m1 * v2[2]) / m1;
                            }
                        }
                    } else {
                        if (m1 != 0.0f) {
                            float cn[3];
                            contact_normal(rv1, n1, a.sc.mu, cn);
                            v1[0] = B0[0].y / m1 - ap1 * cn[0];
                            v1[1] = B0[0].z / m1 - ap1 * cn[1];
                            v1[2] = B0[0].w / m1 - ap1 * cn[2];
                            a1[0] = B1[0].x / m1 - (ap1 * cn[0]) / dt;
                            a1[1] = B1[0].y / m1 - (ap1 * cn[1]) / dt;
                            a1[2] = B1[0].z / m1 - (ap1 * cn[2]) / dt;
                            for (int k = 0; k < 3; k++) v1[k] += a1[k] * dtn;
                        }
                        if (m2 != 0.0f) {
                            float cn[3];
                            contact_normal(rv2, n2, a.sc.mu, cn);
                            v2[0] = B0[1].y / m2 - ap2 * cn[0];
                            v2[1] = B0[1].z / m2 - ap2 * cn[1];
                            v2[2] = B0[1].w / m2 - ap2 * cn[2];
                            a2[0] = B1[1].x / m2 - (ap2 * cn[0]) / dt;
                            a2[1] = B1[1].y / m2 - (ap2 * cn[1]) / dt;
                            a2[2] = B1[1].z / m2 - (ap2 * cn[2]) / dt;
                            for (int k = 0; k < 3; k++) v2[k] += a2[k] * dtn;
                        }
                    }
                } else {
                    if (m1 != 0.0f) body_update(m1, B0[0], B1[0], dtn, v1, a1);
                    if (m2 != 0.0f) body_update(m2, B0[1], B1[1], dtn, v2, a2);
                }
            } else {
                if (m1 != 0.0f) body_update(m1, B0[0], B1[0], dtn, v1, a1);
            }
        }
    }
    // grid BC, phase 2 (phase 1 values are overwritten by the solve for every node the
    // particles read; phase 3 repeats phase 2)
    const int bt = nb.bc_type ? nb.bc_type[nd] : 0;
    if (bt) {
        BCApply bc{bt, nb.bc_val[nd], a.sc.fixed_grid_bcs};
        bool set[3];
        float val[3];
        bc.comps(set, val);
        for (int k = 0; k < 3; k++)
            if (set[k]) {
                v1[k] = val[k]; a1[k] = 0.f;
                v2[k] = val[k]; a2[k] = 0.f;
                vc[k] = val[k];
            }
    }
    nb.gv[nd] = make_float4(m, v1[0], v1[1], v1[2]);
    nb.ga[nd] = make_float4(a1[0], a1[1], a1[2], 0.f);
    if (MULTI) {
        nb.bgv[0][nd] = make_float4(m, v1[0], v1[1], v1[2]);
        nb.bga[0][nd] = make_float4(a1[0], a1[1], a1[2], 0.f);
        nb.bgv[1][nd] = make_float4(m, v2[0], v2[1], v2[2]);
        nb.bga[1][nd] = make_float4(a2[0], a2[1], a2[2], 0.f);
        if (nb.nrm_out[0]) {
            nb.nrm_out[0][nd] = make_float4(n1[0], n1[1], n1[2], 0.f);
            nb.nrm_out[1][nd] = make_float4(-n1[0], -n1[1], -n1[2], 0.f);
        }
    }
    if (keep) {
        nb.out_com[nd] = make_float4(vc[0], vc[1], vc[2], 0.f);
        nb.out_force[nd] = make_float4(A1.x, A1.y, A1.z, 0.f);
    }
    if (nb.active_count) {
        const unsigned mask = __ballot_sync(__activemask(), active);
        if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && mask) atomicAdd(nb.active_count, __popc(mask));
    }
}

void launch_solve(const NodeBufs &nb, const StepArgs &a, bool keep_node_fields, cudaStream_t s)
{
    const unsigned grid = (unsigned)((a.g.nn + 255) / 256);
    if (a.sc.multi_body) {
        k_solve<true><<<grid, 256, 0, s>>>(nb, a, keep_node_fields ? 1 : 0);
        note_launch(1);
    }
    else {
        k_solve<false><<<grid, 256, 0, s>>>(nb, a, keep_node_fields ? 1 : 0);
        note_launch(1);
    }
}

// ---------------------------------------------------------------------------------------
// G2P + particle BCs + update + constitutive + damage + wrap + key

__device__ __forceinline__ float sinf_ref(float x) { return sinf(x); }

// particle BCs, TimeIntegration.cpp:177-296
__device__ __forceinline__ void particle_bc(int type, const float4 &val, float t, float mass, float v[3], float acc[3],
                                            float vg[3], float s[6])
{
    const float w = 2.0f * 3.14159f;
    switch (type) {
    case BC_MP_VX: v[0] = val.x; break;
    case BC_MP_VY: v[0] = 0.f; v[1] = val.x; v[2] = 0.f; break;
    case BC_MP_VZ: v[0] = 0.f; v[1] = 0.f; v[2] = val.x; break;
    case BC_MP_VX_VY: v[0] = val.x; v[1] = val.y; v[2] = 0.f; break;
    case BC_MP_VXSIN: v[0] = val.x * sinf_ref(w * val.y * t); break;
    case BC_MP_VYSIN: v[1] = val.x * sinf_ref(w * val.y * t); vg[1] = 0.f; acc[1] = 0.f; break;
    case BC_MP_SYYSIN:
        s[1] = val.x * sinf_ref(w * val.y * t);
        v[0] = v[1] = v[2] = 0.f;
        vg[0] = vg[1] = vg[2] = 0.f;
        break;
    case BC_MP_FX: acc[0] += val.x / mass; break;
    case BC_MP_FY: acc[0] = 0.f; acc[1] += val.x / mass; break;
    case BC_MP_FZ: acc[2] += val.x / mass; break;
    case BC_MP_FX_FY: acc[0] += val.x / mass; acc[1] += val.y / mass; break;
    case BC_MP_STRESS_XX_YY: s[0] = val.x; s[1] = val.y; break;
    default: break;
    }
}

// move an (offset, cell) pair by delta cells and renormalise the offset into [lp, 1+lp)
__device__ __forceinline__ void renorm(float &o, int &c, float lp)
{
    const float k = floorf(o - lp);
    if (k != 0.0f) {
        o -= k;
        c += (int)k;
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_g2p_update(PView P, long long n, NodeBufs nb, StepArgs a, int track_normals,
                                                    int check_finite, int has_dp)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GridGeom &g = a.g;
    const StepScalars &sc = a.sc;
    const uint32_t info = (uint32_t)P.ii(PF_INFO, i);
    int ci, cj, ck;
    decode_key(P.ii(PF_KEY, i), g, ci, cj, ck);
    float o[3] = {P.f(PF_OX, i), P.f(PF_OY, i), P.f(PF_OZ, i)};
    float Sx[3], Gx[3], Sy[3], Gy[3], Sz[3] = {1.f, 0.f, 0.f}, Gz[3] = {0.f, 0.f, 0.f};
    gimp_axis(o[0], g.lp, Sx, Gx);
    gimp_axis(o[1], g.lp, Sy, Gy);
    int nkz = 1;
    if (g.is3d) {
        gimp_axis(o[2], g.lp, Sz, Gz);
        nkz = (o[2] < 1.0f - g.lp) ? 2 : 3;
    } else {
        ck = 0;
    }
    const int nix = (o[0] < 1.0f - g.lp) ? 2 : 3;
    const int njy = (o[1] < 1.0f - g.lp) ? 2 : 3;
    const int obj = info_obj(info);

    // ---- G2P (Extrapolation.cpp:288-367) ----
    float acc[3] = {0.f, 0.f, 0.f}, vg[3] = {0.f, 0.f, 0.f}, nrm[3] = {0.f, 0.f, 0.f};
    float L[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // L[a][b] = sum v_a dW/dx_b
    for (int kk = 0; kk < nkz; kk++)
        for (int jj = 0; jj < njy; jj++) {
            const float syz = Sy[jj] * Sz[kk], gyz = Gy[jj] * Sz[kk], syg = Sy[jj] * Gz[kk];
            for (int ii = 0; ii < nix; ii++) {
                const long long nd = node_index(ci + ii, cj + jj, ck + kk, g);
                const float4 V = __ldg(&nb.gv[nd]);
                if (V.x == 0.0f) continue;  // nodes without mass are skipped
                float4 Vb, Ab;
                if (!MULTI) {
                    Vb = V;
                    Ab = __ldg(&nb.ga[nd]);
                } else {
                    const int2 b = __ldg(&nb.body[nd]);
                    const int slot = (b.x == obj) ? 0 : ((b.y == obj) ? 1 : -1);
                    if (slot < 0) continue;  // a third body sees nothing from this node
                    Vb = __ldg(&nb.bgv[slot][nd]);
                    Ab = __ldg(&nb.bga[slot][nd]);
                }
                const float w = Sx[ii] * syz;
                const float gx = Gx[ii] * syz * g.inv_h, gy = Sx[ii] * gyz * g.inv_h, gz = Sx[ii] * syg * g.inv_h;
                acc[0] += w * Ab.x; acc[1] += w * Ab.y; acc[2] += w * Ab.z;
                vg[0] += w * Vb.y; vg[1] += w * Vb.z; vg[2] += w * Vb.w;
                L[0][0] += Vb.y * gx; L[0][1] += Vb.y * gy; L[0][2] += Vb.y * gz;
                L[1][0] += Vb.z * gx; L[1][1] += Vb.z * gy; L[1][2] += Vb.z * gz;
                L[2][0] += Vb.w * gx; L[2][1] += Vb.w * gy; L[2][2] += Vb.w * gz;
                if (MULTI && track_normals) {
                    const int2 b = __ldg(&nb.body[nd]);
                    const float4 N = __ldg(&nb.nrm_out[(b.x == obj) ? 0 : 1][nd]);
                    nrm[0] += w * N.x; nrm[1] += w * N.y; nrm[2] += w * N.z;
                }
            }
        }

    Constit c;
    c.r[0] = L[0][0];
    c.r[1] = L[1][1];
    c.r[2] = L[2][2];
    c.r[3] = 0.5f * (L[1][0] + L[0][1]);
    c.r[4] = 0.5f * (L[2][1] + L[1][2]);
    c.r[5] = 0.5f * (L[2][0] + L[0][2]);
    float rho = P.f(PF_RHO, i);
    const float rho_rate = -rho * (L[0][0] + L[1][1] + L[2][2]);
    float v[3] = {P.f(PF_VX, i), P.f(PF_VY, i), P.f(PF_VZ, i)};
#pragma unroll
    for (int k = 0; k < 6; k++) {
        c.s[k] = P.f(PF_S0 + k, i);
        c.e[k] = P.f(PF_E0 + k, i);
    }
    const float mass = P.f(PF_MASS, i);
    const int bct = info_bc(info);
    float4 bcv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (bct) bcv = __ldg(&a.pbc_val[P.ii(PF_PID, i)]);

    // ---- particle BC, phase 4 ----
    if (bct) particle_bc(bct, bcv, sc.t_bc, mass, v, acc, vg, c.s);

    // ---- update (TimeIntegration.cpp:11-117) ----
    const float dt = sc.dt;
    rho += rho_rate * dt;
    if (!(info & INFO_HOLD)) {
        v[0] = v[0] + (acc[0] - sc.damping * v[0]) * dt;
        v[1] = v[1] + (acc[1] - sc.damping * v[1]) * dt;
        if (g.is3d) v[2] = v[2] + (acc[2] - sc.damping * v[2]) * dt;
        o[0] += vg[0] * dt * g.inv_h;
        o[1] += vg[1] * dt * g.inv_h;
        if (g.is3d) o[2] += vg[2] * dt * g.inv_h;
    }
#pragma unroll
    for (int k = 0; k < 6; k++) c.e[k] += c.r[k] * dt;
    const DevMaterial &M = a.mats[info_mat(info)];
    if (has_dp) {
        c.eqps = P.f(PF_EQPS, i);
#pragma unroll
        for (int k = 0; k < 6; k++) c.ep[k] = P.f(PF_EP0 + k, i);
        c.dmg = P.f(PF_DMG, i);
        c.smax = P.f(PF_SMAX, i);
    } else {
        c.eqps = 0.f;
        c.dmg = 0.f;
        c.smax = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) c.ep[k] = 0.f;
    }
    c.mass = mass;
    c.rho = rho;
    c.v[0] = v[0]; c.v[1] = v[1]; c.v[2] = v[2];
    if (!(info & INFO_RIGID)) constitutive_update(c, M, dt, g.is3d);

    // ---- periodic wrap (TimeIntegration.cpp:80-108) and new cell ----
    int cc[3] = {ci, cj, ck};
    const int naxes = g.is3d ? 3 : 2;
    for (int ax = 0; ax < naxes; ax++) {
        renorm(o[ax], cc[ax], g.lp);
        const float X = (float)cc[ax] + o[ax];
        int sh = 0;
        float sf = 0.f;
        if (X > g.wrap_hi[ax]) { sh = g.wrap_shift_int[ax]; sf = g.wrap_shift_frac[ax]; }
        if (X + (float)sh + sf < 1.0f) { sh -= g.wrap_shift_int[ax]; sf -= g.wrap_shift_frac[ax]; }
        if (sh != 0 || sf != 0.f) {
            cc[ax] += sh;
            o[ax] += sf;
            renorm(o[ax], cc[ax], g.lp);
        }
    }
    const int lim[3] = {g.ncx - 2, g.ncy - 2, g.ncz - 2};
    bool bad = false;
    for (int ax = 0; ax < naxes; ax++) {
        if (cc[ax] < 0) { cc[ax] = 0; bad = true; }
        if (cc[ax] > lim[ax]) { cc[ax] = lim[ax]; bad = true; }
    }
    if (bad) atomicOr(a.status, ERR_RANGE);
    const int nkey = cc[0] + cc[1] * g.ncx + (g.is3d ? cc[2] * g.ncx * g.ncy : 0);

    // ---- particle BC, phase 5 ----
    if (bct) particle_bc(bct, bcv, sc.t_bc, mass, v, acc, vg, c.s);

    if (check_finite) {
        bool fin = isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]) && isfinite(rho);
#pragma unroll
        for (int k = 0; k < 6; k++) fin = fin && isfinite(c.s[k]);
        if (!fin) atomicOr(a.status, ERR_NONFINITE);
    }

    // ---- write back ----
    P.f(PF_OX, i) = o[0];
    P.f(PF_OY, i) = o[1];
    if (g.is3d) P.f(PF_OZ, i) = o[2];
    P.ii(PF_KEY, i) = nkey;
    P.f(PF_VX, i) = v[0];
    P.f(PF_VY, i) = v[1];
    P.f(PF_VZ, i) = v[2];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        P.f(PF_S0 + k, i) = c.s[k];
        P.f(PF_E0 + k, i) = c.e[k];
    }
    P.f(PF_RHO, i) = rho;
    if (info & INFO_INIT_VOL) P.ii(PF_INFO, i) = (int)(info & ~INFO_INIT_VOL);
    if (has_dp) {
        P.f(PF_EQPS, i) = c.eqps;
#pragma unroll
        for (int k = 0; k < 6; k++) P.f(PF_EP0 + k, i) = c.ep[k];
        P.f(PF_DMG, i) = c.dmg;
        P.f(PF_SMAX, i) = c.smax;
    }
    if (track_normals) {
        P.f(PF_NX, i) = nrm[0];
        P.f(PF_NY, i) = nrm[1];
        P.f(PF_NZ, i) = nrm[2];
    }
}

void launch_g2p_update(const PView &p, long long n, const NodeBufs &nb, const StepArgs &a, bool track_normals,
                       bool check_finite, bool has_dp, int block, cudaStream_t s)
{
    (void)block;
    if (n == 0) return;
    const int B = 256;
    const unsigned grid = (unsigned)((n + B - 1) / B);
    if (a.sc.multi_body)
        k_g2p_update<true><<<grid, B, 0, s>>>(p, n, nb, a, track_normals ? 1 : 0, check_finite ? 1 : 0, has_dp ? 1 : 0);
    else
        k_g2p_update<false><<<grid, B, 0, s>>>(p, n, nb, a, 0, check_finite ? 1 : 0, has_dp ? 1 : 0);
    note_launch(1);
}

// ---------------------------------------------------------------------------------------
// Body slots (Extrapolation.cpp:191-208).  The reference assigns each node's two body slots
// to the objects of the first particles it visits in its 4x4x4 cell window (cells in
// increasing linear id, particles in sorted order within a cell), using the cell table of
// the last sort.  Here a per-(cell, object) table holds the smallest particle id of that
// object in the cell (the within-cell order both sides use) plus a rigid bit per object,
// and each node scans its window in the reference's order.

constexpr int NO_PARTICLE = 0x7fffffff;

__global__ void k_body_tables(PView P, long long n, StepArgs a, int *cell_min, int nbody, const int *refkeys)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t info = (uint32_t)P.ii(PF_INFO, i);
    const int obj = info_obj(info);
    int rk;
    if (refkeys) {
        rk = refkeys[P.ii(PF_PID, i)];
    } else {
        // the reference's binning key from the current position (TimeIntegration.cpp:110-115)
        int ci, cj, ck;
        decode_key(P.ii(PF_KEY, i), a.g, ci, cj, ck);
        const int ix = (int)((float)ci + P.f(PF_OX, i) - 0.25f);
        const int iy = (int)((float)cj + P.f(PF_OY, i) - 0.25f);
        const int iz = a.g.is3d ? (int)((float)ck + P.f(PF_OZ, i) - 0.25f) : 0;
        rk = ix + iy * a.g.ncx + iz * a.g.ncx * a.g.ncy;
    }
    if (rk < 0 || rk >= a.g.nc) return;
    atomicMin(&cell_min[(long long)rk * (nbody + 1) + obj], P.ii(PF_PID, i));
    if (info & INFO_RIGID) atomicOr(&cell_min[(long long)rk * (nbody + 1) + nbody], 1 << obj);
}

__global__ void k_body_clear(int *cell_min, long long nc, int nbody)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int *row = cell_min + c * (nbody + 1);
    for (int b = 0; b < nbody; b++) row[b] = NO_PARTICLE;
    row[nbody] = 0;
}

void launch_body_tables(const PView &p, long long n, const StepArgs &a, int *cell_min, int nbody,
                        const int *refkeys, cudaStream_t s)
{
    k_body_clear<<<(unsigned)((a.g.nc + 255) / 256), 256, 0, s>>>(cell_min, a.g.nc, nbody);
    note_launch(1);
    if (n == 0) return;
    k_body_tables<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, n, a, cell_min, nbody, refkeys);
    note_launch(1);
}

__global__ void k_body_assign(NodeBufs nb, GridGeom g, const int *cell_min, int nbody, const int *nidx_x,
                              const int *nidx_y, const int *nidx_z)
{
    const long long nd = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= g.nn) return;
    const int i = (int)(nd % g.nx);
    const int j = (int)((nd / g.nx) % g.ny);
    const int k = (int)(nd / ((long long)g.nx * g.ny));
    const int cx = nidx_x[i], cy = nidx_y[j], cz = g.is3d ? nidx_z[k] : 0;
    const int stride = nbody + 1;
    int b0 = -1, b1 = -1;
    int rig = 0;  // OR of rigid bits over the window
    const int kmin = g.is3d ? -2 : 0, kmax = g.is3d ? 2 : 1;
    for (int kk = kmin; kk < kmax; kk++)
        for (int jj = -2; jj < 2; jj++)
            for (int ii = -2; ii < 2; ii++) {
                const long long c = (long long)(cx + ii) + (long long)(cy + jj) * g.ncx + (long long)(cz + kk) * g.ncx * g.ncy;
                if (c >= g.nc || c < 0) continue;
                const int *row = cell_min + c * stride;
                rig |= row[nbody];
                if (b1 != -1) continue;
                // first particle of the cell, and first one whose object differs from b0
                int first = -1, fpid = NO_PARTICLE, other = -1, opid = NO_PARTICLE;
                for (int b = 0; b < nbody; b++) {
                    const int pid = row[b];
                    if (pid == NO_PARTICLE) continue;
                    if (pid < fpid) { fpid = pid; first = b; }
                }
                if (first < 0) continue;
                if (b0 == -1) b0 = first;
                for (int b = 0; b < nbody; b++) {
                    const int pid = row[b];
                    if (b == b0 || pid == NO_PARTICLE) continue;
                    if (pid < opid) { opid = pid; other = b; }
                }
                if (other >= 0) b1 = other;
            }
    nb.body[nd] = make_int2(b0, b1);
    unsigned char hr = 0;
    if (b0 >= 0 && (rig >> b0) & 1) hr |= 1;
    if (b1 >= 0 && (rig >> b1) & 1) hr |= 2;
    nb.has_rigid[nd] = hr;
}

void launch_body_assign(const NodeBufs &nb, const StepArgs &a, const int *cell_min, int nbody, const int *nidx_x,
                        const int *nidx_y, const int *nidx_z, cudaStream_t s)
{
    k_body_assign<<<(unsigned)((a.g.nn + 255) / 256), 256, 0, s>>>(nb, a.g, cell_min, nbody, nidx_x, nidx_y, nidx_z);
    note_launch(1);
}

// ---------------------------------------------------------------------------------------
// FP64 conservation sums: mass, momentum, kinetic energy, strain energy

__global__ void k_stats(PView P, long long n, StepArgs a, double *out)
{
    __shared__ double sh[8][8];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double m = P.f(PF_MASS, i);
        const double vx = P.f(PF_VX, i), vy = P.f(PF_VY, i), vz = P.f(PF_VZ, i);
        acc[0] += m;
        acc[1] += m * vx;
        acc[2] += m * vy;
        acc[3] += m * vz;
        acc[4] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        const double V = m / (double)P.f(PF_RHO, i);
        double se = 0.0;
        for (int k = 0; k < 3; k++) se += (double)P.f(PF_S0 + k, i) * P.f(PF_E0 + k, i);
        for (int k = 3; k < 6; k++) se += 2.0 * (double)P.f(PF_S0 + k, i) * P.f(PF_E0 + k, i);
        acc[5] += 0.5 * V * se;
    }
    for (int k = 0; k < 6; k++) {
        double v = acc[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffff, v, off);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[w][threadIdx.x];
        atomicAdd(&out[threadIdx.x], v);
    }
}

void launch_stats(const PView &p, long long n, const StepArgs &a, double *out8, cudaStream_t s)
{
    cudaMemsetAsync(out8, 0, 8 * sizeof(double), s);
    if (n == 0) return;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_stats<<<(unsigned)blocks, 256, 0, s>>>(p, n, a, out8);
    note_launch(1);
}

}  // namespace gy
