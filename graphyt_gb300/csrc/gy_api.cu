// gy_api.cu -- host runtime behind the C ABI (include/graphyt_gpu.h).
//
// Owns the device state of one simulation, converts the reference's host-side model
// (Nodes, MaterialPoints, MaterialModels, Parameters, Solver) into the GPU layout and
// sequences the kernels of one step on the handle's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/graphyt_gpu.h"
#include "gy_kernels.cuh"

using namespace gy;

// Everything a step enqueues is fixed by this variant; the per-step scalars live in device
// memory, so one captured graph per variant replays any step of that variant.
struct StepVariant {
    int cur;       // slab read this step
    int sk;        // sorted-key buffer written by this step's sort (the other one is read)
    int sort;      // 0 none, 1 incremental, 2 full
    int tables;    // 0 none, 1 rebuild body tables, 2 rebuild from the initial keys
    bool operator==(const StepVariant &o) const
    {
        return cur == o.cur && sk == o.sk && sort == o.sort && tables == o.tables;
    }
};

struct StepGraph {
    StepVariant v;
    cudaGraphExec_t exec;
    long long launches;  // kernels in the graph
};


struct gy_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // grid (Nodes)
    double L[3] = {0, 0, 0}, h = 0, psep = 0;
    int nx = 0, ny = 0, nz = 0;
    long long nn = 0;
    GridGeom g{};
    std::vector<int> nidx[3];

    // host staging, insertion order (MaterialPoints)
    std::vector<double> pos, vel, stress, dmg, temp;
    std::vector<double> flaw;        // Grady-Kipp activation strain scale (1: the reference's e_min)
    std::vector<int> mat, obj, pbc_type;
    std::vector<double> pbc_val;
    std::vector<unsigned char> hold;
    std::vector<int> key0;           // uploaded cell key by particle id
    std::vector<float> off0;         // uploaded FP32 offsets by particle id (3 per particle)
    std::vector<unsigned char> nbc_type;
    std::vector<float> nbc_val;
    bool any_node_bc = false;

    // model
    std::vector<gy_material> mats;
    gy_params prm{};
    double dt = 0.0;
    bool initialized = false;
    gy_options opt{1, 0, 1, 0, 0, 0, 3};
    std::vector<int> slot_obj;       // dense object slot -> objectID
    bool multi = false, has_dp = false;
    int nbody = 1;

    // device particle state
    long long n = 0, cap = 0;
    float *slab[2] = {nullptr, nullptr};
    int cur = 0;
    int *d_perm = nullptr;
    int *d_seg = nullptr, *d_nseg = nullptr;   // non-empty cell-block segments; two counts, by slab parity
    int persist_grid = 1;
    int g2p_grid = 1;
    SortScratch ws{};
    void *sort_mem = nullptr;
    ResortScratch rs{};
    void *resort_mem = nullptr;
    int *skey_buf[2] = {nullptr, nullptr};  // sorted keys of the last sort and its successor
    int *d_blk_first = nullptr;             // first position of each cell block at the last sort
    int sk = 0;
    bool resort_valid = false;              // slab order = order of the sort in skey_buf[sk]
    StepScalars *d_sc = nullptr;            // this step's scalars (device)
    static constexpr int kRing = 32;        // pinned staging slots for the per-step scalars
    StepScalars *h_ring = nullptr;
    struct Readback {
        double part[STATS_SLOTS * 8];
        int flags[4];
    } *h_rb = nullptr;                      // pinned: the step's sums and status words
    cudaEvent_t ring_ev[kRing] = {};
    bool ring_busy[kRing] = {};
    long long ring_pos = 0;
    std::vector<StepGraph> graphs;          // captured steps, one per StepVariant
    float4 *d_pbc_val = nullptr;
    float *d_flaw = nullptr;                // flaw scale by insertion index, or null (every scale 1)
    // learned Drucker-Prager surrogate: training-pair log, deferred particles, parameters
    float *d_dplog = nullptr;               // [cap][16] inputs then [cap][7] targets
    unsigned int *d_dplog_n = nullptr;
    unsigned int dplog_cap = 0;
    int dplog_every = 1;
    bool dplog_on = false;
    float4 *d_pend = nullptr;               // [n][2] deferred particles
    unsigned int *d_pend_n = nullptr;
    float *d_surr = nullptr;                // gy_mlp_param_count() floats
    unsigned long long *d_surr_counts = nullptr;  // kept predictions, fallbacks
    float surr_tol = 1e-4f;
    bool surr_on = false;
    int *d_refkey0 = nullptr;
    DevMaterial *d_mats = nullptr;
    int *d_status = nullptr;
    double *d_stats = nullptr;              // STATS_SLOTS x 8 conservation partials
    float4 *d_therm = nullptr;              // (T, grad T) by insertion index, once a temperature is set
    float2 *d_tnode = nullptr;              // node (T sum, T rate), zero between steps
    bool thermal = false;                   // run the heat conduction kernels
    void *d_tset = nullptr;                 // scratch of gy_set_particle_temp between steps
    size_t tset_bytes = 0;
    bool stats_fresh = false;               // d_stats holds the sums of the current state
    double mass_total = 0.0;                // FP64 total mass (no step changes a mass)

    // device node state
    NodeBufs nb{};
    void *node_mem = nullptr;
    int *d_cell_min = nullptr;
    int *d_nidx[3] = {nullptr, nullptr, nullptr};

    // stepping
    double t_prev = 0.0;
    long long steps = 0;
    long long since_sort = 1 << 30;
    bool tables_valid = false;
    bool phase_timing = false;
    cudaEvent_t ev[6] = {};
    std::vector<cudaEvent_t> tev;   // phase-timing pool: 5 events per timed step
    long long tev_used = 0;
};

static constexpr long long kMaxTimedSteps = 4096;

namespace {

gy_status fail(gy_solver *h, gy_status code, const std::string &msg)
{
    if (h) h->err = msg;
    return code;
}

#define CK(h, call)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(h, e_ == cudaErrorMemoryAllocation ? GY_ERR_NOMEM : GY_ERR_CUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(e_));               \
    } while (0)

template <class T> gy_status dalloc(gy_solver *h, T **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T) + 16);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(h, GY_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return GY_OK;
}

PView pview(gy_solver *h, int which) { return PView{h->slab[which], h->cap}; }

void drop_graphs(gy_solver *h)
{
    for (auto &gr : h->graphs)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    h->graphs.clear();
}

void free_device(gy_solver *h)
{
    drop_graphs(h);
    if (h->h_ring) cudaFreeHost(h->h_ring);
    h->h_ring = nullptr;
    if (h->h_rb) cudaFreeHost(h->h_rb);
    h->h_rb = nullptr;
    for (int k = 0; k < gy_solver::kRing; k++) {
        if (h->ring_ev[k]) cudaEventDestroy(h->ring_ev[k]);
        h->ring_ev[k] = nullptr;
        h->ring_busy[k] = false;
    }
    void *ptrs[] = {h->slab[0], h->slab[1], h->d_perm, h->d_seg, h->d_nseg, h->sort_mem, h->resort_mem, h->d_pbc_val,
                    h->d_refkey0, h->d_mats, h->d_status, h->d_stats, h->node_mem, h->d_cell_min,
                    h->d_nidx[0], h->d_nidx[1], h->d_nidx[2], h->d_sc, h->d_therm, h->d_tnode, h->d_tset, h->d_flaw,
                    h->d_dplog, h->d_dplog_n, h->d_pend, h->d_pend_n, h->d_surr, h->d_surr_counts};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    h->d_sc = nullptr;
    h->d_therm = nullptr;
    h->d_tnode = nullptr;
    h->d_tset = nullptr;
    h->tset_bytes = 0;
    h->thermal = false;
    h->slab[0] = h->slab[1] = nullptr;
    h->d_perm = h->d_seg = h->d_nseg = nullptr;
    h->sort_mem = nullptr;
    h->resort_mem = nullptr;
    h->skey_buf[0] = h->skey_buf[1] = nullptr;
    h->d_blk_first = nullptr;
    h->d_pbc_val = nullptr;
    h->d_flaw = nullptr;
    h->d_dplog = nullptr;
    h->d_dplog_n = nullptr;
    h->dplog_cap = 0;
    h->dplog_on = false;
    h->d_pend = nullptr;
    h->d_pend_n = nullptr;
    h->d_surr = nullptr;
    h->d_surr_counts = nullptr;
    h->surr_on = false;
    h->d_refkey0 = nullptr;
    h->d_mats = nullptr;
    h->d_status = nullptr;
    h->d_stats = nullptr;
    h->node_mem = nullptr;
    h->d_cell_min = nullptr;
    for (int a = 0; a < 3; a++) h->d_nidx[a] = nullptr;
}

bool valid_index(const gy_solver *h, int64_t i) { return i >= 0 && i < (int64_t)h->mat.size(); }

}  // namespace

extern "C" {

int gy_abi_version(void) { return GY_ABI_VERSION; }

const char *gy_last_error(const gy_solver *h) { return h ? h->err.c_str() : "null handle"; }

gy_status gy_create(const gy_grid_desc *grid, int device, gy_solver **out)
{
    if (!grid || !out) return GY_ERR_ARG;
    *out = nullptr;
    const double h = grid->cellsize;
    if (!(h > 0) || !(grid->psep > 0) || grid->L[0] <= 0 || grid->L[1] <= 0 || grid->L[2] < 0) return GY_ERR_ARG;
    // Nodes.cpp:12 rounds numNodes while :71-73 truncate Nx, Ny, Nz
    const double nn_r = std::round((1.0 + grid->L[0] / h) * (1.0 + grid->L[1] / h) * (1.0 + grid->L[2] / h));
    const int nx = (int)(1.0 + grid->L[0] / h), ny = (int)(1.0 + grid->L[1] / h), nz = (int)(1.0 + grid->L[2] / h);
    if ((double)nx * ny * nz != nn_r) return GY_ERR_ARG;
    if ((double)nx * ny * nz >= 2147483647.0) return GY_ERR_UNSUPPORTED;  // 32-bit node indices
    const bool is3d = nz > 1;
    if (nx < 6 || ny < 6 || (is3d && nz < 6)) return GY_ERR_ARG;  // the periodic fold pairs 3 layers per side
    if (grid->psep > h) return GY_ERR_UNSUPPORTED;                  // 3-node stencil needs psep/2 <= h/2
    gy_solver *s = new gy_solver();
    s->device = device;
    if (device >= 0) {
        if (cudaSetDevice(device) != cudaSuccess) {
            delete s;
            return GY_ERR_CUDA;
        }
    } else {
        cudaGetDevice(&s->device);
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return GY_ERR_CUDA;
    }
    for (int i = 0; i < 6; i++) cudaEventCreate(&s->ev[i]);
    for (int a = 0; a < 3; a++) s->L[a] = grid->L[a];
    s->h = h;
    s->psep = grid->psep;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->nn = (long long)nx * ny * nz;
    GridGeom &g = s->g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.ncx = nx - 1; g.ncy = ny - 1; g.ncz = is3d ? nz - 1 : 1;
    g.nn = s->nn;
    g.nc = (long long)g.ncx * g.ncy * g.ncz;
    g.nbx = (g.ncx + CB - 1) / CB;
    g.nby = (g.ncy + CB - 1) / CB;
    g.nbz = (g.ncz + CB - 1) / CB;
    g.nnbx = (nx + 3) / 4;
    g.nnby = (ny + 3) / 4;
    g.nnbz = (nz + 3) / 4;
    g.nnb = (long long)g.nnbx * g.nnby * g.nnbz;
    g.div_nbx = ((1ULL << 39) + g.nbx - 1) / g.nbx;
    g.div_nby = ((1ULL << 39) + g.nby - 1) / g.nby;
    if ((long long)g.nbx * g.nby * g.nbz >= (1LL << 25) || g.nbx >= (1 << 14) || g.nby >= (1 << 14)) {
        cudaStreamDestroy(s->stream);
        delete s;
        return GY_ERR_UNSUPPORTED;  // cell keys must fit in 31 bits
    }
    g.h = (float)h;
    g.inv_h = (float)(1.0 / h);
    g.lp = (float)(0.5 * grid->psep / h);
    g.inv_l = (float)(1.0 / (double)g.lp);
    g.inv_2l = (float)(0.5 / (double)g.lp);
    g.inv_4l = (float)(0.25 / (double)g.lp);
    g.is3d = is3d ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        const double W = grid->L[a] / h - 2.0;  // the wrap limit L - 2h in cells
        const double shift = 1.0 - W;           // x > L-2h:  x -> h + (x - (L-2h))
        g.wrap_hi[a] = (float)W;
        g.wrap_shift_int[a] = (int)std::floor(shift);
        g.wrap_shift_frac[a] = (float)(shift - std::floor(shift));
    }
    // node cell index as extrapToNodes derives it from the node position (Extrapolation.cpp:43-45)
    const int dims[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++) {
        s->nidx[a].resize(dims[a]);
        for (int i = 0; i < dims[a]; i++) {
            const double p = i * h;
            s->nidx[a][i] = (int)((p - 0.0) / h);
        }
    }
    s->nbc_type.assign((size_t)s->nn, 0);
    s->nbc_val.assign((size_t)s->nn * 4, 0.0f);
    *out = s;
    return GY_OK;
}

gy_status gy_destroy(gy_solver *h)
{
    if (!h) return GY_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_device(h);
    for (int i = 0; i < 6; i++)
        if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GY_OK;
}

gy_status gy_grid_dims(const gy_solver *h, int *nxyz, int64_t *num_nodes)
{
    if (!h) return GY_ERR_ARG;
    if (nxyz) { nxyz[0] = h->nx; nxyz[1] = h->ny; nxyz[2] = h->nz; }
    if (num_nodes) *num_nodes = h->nn;
    return GY_OK;
}

gy_status gy_add_particles(gy_solver *h, int64_t n, const double *pos3, const int *mat, const int *obj)
{
    if (!h || n < 0 || (n > 0 && !pos3)) return GY_ERR_ARG;
    if (h->initialized) return fail(h, GY_ERR_STATE, "particles must be added before gy_initialize");
    if ((int64_t)h->mat.size() + n > (int64_t)0x7fffffff) return fail(h, GY_ERR_ARG, "too many particles");
    for (int64_t i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) {
            h->pos.push_back(pos3[3 * i + k]);
            h->vel.push_back(0.0);
        }
        for (int k = 0; k < 6; k++) h->stress.push_back(0.0);
        h->dmg.push_back(0.0);
        h->flaw.push_back(1.0);
        h->temp.push_back(0.0);
        h->mat.push_back(mat ? mat[i] : 0);
        h->obj.push_back(obj ? obj[i] : 0);
        h->pbc_type.push_back(0);
        for (int k = 0; k < 4; k++) h->pbc_val.push_back(0.0);
        h->hold.push_back(0);
    }
    return GY_OK;
}

#define PRE_INIT(h)                                                                                   \
    do {                                                                                              \
        if (!(h)) return GY_ERR_ARG;                                                                  \
        if ((h)->initialized) return fail(h, GY_ERR_STATE, "particle/node setters must precede gy_initialize"); \
    } while (0)

gy_status gy_set_particle_vel(gy_solver *h, int64_t count, const int64_t *idx, const double *v)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        for (int k = 0; k < 3; k++) h->vel[3 * idx[q] + k] = v[3 * q + k];
    }
    return GY_OK;
}

gy_status gy_set_particle_stress(gy_solver *h, int64_t count, const int64_t *idx, const double *s6)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        for (int k = 0; k < 6; k++) h->stress[6 * idx[q] + k] = s6[6 * q + k];
    }
    return GY_OK;
}

gy_status gy_set_particle_damage(gy_solver *h, int64_t count, const int64_t *idx, const double *d)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        h->dmg[idx[q]] = d[q];
    }
    return GY_OK;
}

gy_status gy_set_particle_flaw(gy_solver *h, int64_t count, const int64_t *idx, const double *w)
{
    PRE_INIT(h);
    if (count < 0 || (count > 0 && (!idx || !w))) return GY_ERR_ARG;
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        if (!(w[q] > 0.0) || !std::isfinite(w[q])) return fail(h, GY_ERR_ARG, "flaw scale must be positive and finite");
        h->flaw[idx[q]] = w[q];
    }
    return GY_OK;
}

gy_status gy_hold_particles(gy_solver *h, int64_t count, const int64_t *idx)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        h->hold[idx[q]] = 1;
    }
    return GY_OK;
}

gy_status gy_set_particle_bc(gy_solver *h, int64_t count, const int64_t *idx, const int *type, const double *val4)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        if (type[q] < 0 || type[q] > 255) return fail(h, GY_ERR_ARG, "BC type out of range");
        h->pbc_type[idx[q]] = type[q];
        for (int k = 0; k < 4; k++) h->pbc_val[4 * idx[q] + k] = val4[4 * q + k];
    }
    return GY_OK;
}

// Device buffers of the heat conduction terms; T starts from the host values.
static gy_status enable_thermal(gy_solver *h)
{
    if (h->d_therm) return GY_OK;
    gy_status st;
    if ((st = dalloc(h, &h->d_therm, h->cap))) return st;
    if ((st = dalloc(h, &h->d_tnode, h->nn))) return st;
    std::vector<float4> th((size_t)h->cap, make_float4(0.f, 0.f, 0.f, 0.f));
    for (long long i = 0; i < h->n; i++) th[i].x = (float)h->temp[i];
    CK(h, cudaMemcpyAsync(h->d_therm, th.data(), (size_t)h->cap * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemsetAsync(h->d_tnode, 0, (size_t)h->nn * sizeof(float2), h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return GY_OK;
}

gy_status gy_set_particle_temp(gy_solver *h, int64_t count, const int64_t *idx, const double *T)
{
    if (!h || count < 0 || (count > 0 && (!idx || !T))) return GY_ERR_ARG;
    bool any = false;
    for (int64_t q = 0; q < count; q++) {
        if (!valid_index(h, idx[q])) return fail(h, GY_ERR_ARG, "particle index out of range");
        any = any || T[q] != 0.0;
    }
    if (!h->initialized) {
        for (int64_t q = 0; q < count; q++) h->temp[idx[q]] = T[q];
        return GY_OK;
    }
    // between steps: the device copy is authoritative once it exists
    if (!h->d_therm && !any) return GY_OK;  // every temperature is still zero
    cudaSetDevice(h->device);
    gy_status st;
    if ((st = enable_thermal(h))) return st;
    if (count == 0) return GY_OK;
    std::vector<int> ids((size_t)count);
    std::vector<float> tv((size_t)count);
    for (int64_t q = 0; q < count; q++) {
        ids[q] = (int)idx[q];
        tv[q] = (float)T[q];
    }
    // a scratch kept across calls (scripts reset temperatures every step); the copies are
    // synchronous with respect to the host buffers, the kernel runs in stream order
    const size_t need = (size_t)count * (sizeof(int) + sizeof(float));
    if (need > h->tset_bytes) {
        CK(h, cudaStreamSynchronize(h->stream));
        if (h->d_tset) cudaFree(h->d_tset);
        h->d_tset = nullptr;
        h->tset_bytes = 0;
        CK(h, cudaMalloc(&h->d_tset, need));
        h->tset_bytes = need;
    }
    int *d_ids = static_cast<int *>(h->d_tset);
    float *d_t = reinterpret_cast<float *>(d_ids + count);
    CK(h, cudaMemcpyAsync(d_ids, ids.data(), (size_t)count * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(d_t, tv.data(), (size_t)count * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    launch_thermal_set(h->d_therm, d_ids, d_t, (int)count, h->n, h->stream);
    // the host vectors die on return and the next call may rewrite the scratch
    const cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(h, GY_ERR_CUDA, std::string("temperature upload: ") + cudaGetErrorString(e));
    if (!h->thermal) {
        h->thermal = true;
        drop_graphs(h);  // the step now carries the thermal kernels
    }
    return GY_OK;
}

gy_status gy_set_node_bc(gy_solver *h, int64_t count, const int64_t *nodes, const int *type, const double *val4)
{
    PRE_INIT(h);
    for (int64_t q = 0; q < count; q++) {
        const int64_t nd = nodes[q];
        if (nd < 0 || nd >= h->nn) return fail(h, GY_ERR_ARG, "node index out of range");
        if (type[q] < 0 || type[q] > 255) return fail(h, GY_ERR_ARG, "BC type out of range");
        h->nbc_type[nd] = (unsigned char)type[q];
        for (int k = 0; k < 4; k++) h->nbc_val[4 * nd + k] = (float)val4[4 * q + k];
        if (type[q]) h->any_node_bc = true;
    }
    return GY_OK;
}

static DevMaterial to_dev(const gy_material &m)
{
    DevMaterial d{};
    d.K = (float)m.bulkMod;
    d.G = (float)m.shearMod;
    d.rho0 = (float)m.density;
    d.viscosity = (float)m.viscosity;
    d.yield = (float)m.yieldStress;
    d.cohesion = (float)m.cohesion;
    d.crit_strain = (float)m.criticalStrain;
    // Drucker-Prager cone (ConstitutiveModels.cpp:247-295, pi as 3.14159)
    const double phi = m.phi * 3.14159 / 180.0, psi = m.psi * 3.14159 / 180.0;
    const double eta = 6.0 * std::sin(phi) / (std::sqrt(3.0) * (3.0 - std::sin(phi)));
    const double xi = 6.0 * std::cos(phi) / (std::sqrt(3.0) * (3.0 - std::sin(phi)));
    const double etab = (phi == psi) ? eta : 6.0 * std::sin(psi) / (std::sqrt(3.0) * (3.0 - std::sin(psi)));
    d.eta = (float)eta;
    d.xi = (float)xi;
    d.eta_bar = (float)etab;
    // Grady-Kipp (DamageModels.cpp:96-106): alpha = 8 pi Cg^3 k / ((m+1)(m+2)(m+3)) overflows
    // FP32, so ((m+3)/3) alpha^(1/3) is formed in FP64 here
    const double mm = m.damageM;
    const double alpha = (8.0 * 3.14159 * m.Cg * m.Cg * m.Cg * m.damageK) / ((mm + 1.0) * (mm + 2.0) * (mm + 3.0));
    d.gk_m = (float)mm;
    d.gk_rate_coef = (float)(((mm + 3.0) / 3.0) * std::pow(alpha, 1.0 / 3.0));
    d.gk_logk = (float)std::log(m.damageK > 0 ? m.damageK : 1e-300);
    d.turb_stress = (float)m.turbStress;
    d.k_th = (float)m.thermalConductivity;
    d.c_th = (float)m.specificHeatCapacity;
    d.phi_deg = (float)m.phi;
    d.model = m.model;
    d.rigid = m.isRigid ? 1 : 0;
    d.damage = m.isDamage ? 1 : 0;
    d.damage_model = m.damageModel;
    return d;
}

static gy_status alloc_nodes(gy_solver *h)
{
    const long long nn = h->nn;
    // node buffers in one allocation of float4 rows
    int rows = 4;                    // acc0, acc1, gv, ga
    if (h->opt.keep_node_fields) rows += 2;
    if (h->multi) rows += 2 * 3 + 2;  // bacc0, bacc1, bnrm per slot; bgv, bga of slot 1 (slot 0's are gv, ga)
    if (h->multi && h->opt.track_normals) rows += 2;
    size_t bytes = (size_t)rows * nn * sizeof(float4);
    size_t extra = 0;
    const long long ncb = (long long)h->g.nbx * h->g.nby * h->g.nbz;  // cell blocks
    if (h->multi)
        extra = (size_t)nn * sizeof(int2) + (size_t)nn + 64 + (size_t)(ncb + h->g.nnb) * sizeof(int) + 64;
    extra += (size_t)(2 * h->g.nnb + 16) * sizeof(int) + 64;
    if (h->any_node_bc) extra += (size_t)nn * sizeof(float4) + (size_t)nn + 64;
    char *mem = nullptr;
    cudaError_t e = cudaMalloc((void **)&mem, bytes + extra + 4096);
    if (e != cudaSuccess) return fail(h, GY_ERR_NOMEM, std::string("node buffers: ") + cudaGetErrorString(e));
    h->node_mem = mem;
    CK(h, cudaMemsetAsync(mem, 0, bytes + extra + 4096, h->stream));
    float4 *f4 = (float4 *)mem;
    NodeBufs &nb = h->nb;
    nb = NodeBufs{};
    nb.acc0 = f4; f4 += nn;
    nb.acc1 = f4; f4 += nn;
    nb.gv = f4; f4 += nn;
    nb.ga = f4; f4 += nn;
    if (h->opt.keep_node_fields) {
        nb.out_com = f4; f4 += nn;
        nb.out_force = f4; f4 += nn;
    }
    if (h->multi) {
        for (int b = 0; b < 2; b++) {
            nb.bacc0[b] = f4; f4 += nn;
            nb.bacc1[b] = f4; f4 += nn;
            nb.bnrm[b] = f4; f4 += nn;
        }
        nb.bgv[0] = nb.gv;  // the solve stores slot 0's velocity and acceleration as the node's
        nb.bga[0] = nb.ga;
        nb.bgv[1] = f4; f4 += nn;
        nb.bga[1] = f4; f4 += nn;
        if (h->opt.track_normals) {
            nb.nrm_out[0] = f4; f4 += nn;
            nb.nrm_out[1] = f4; f4 += nn;
        }
    }
    char *c = (char *)f4;
    nb.flags = (int *)c;
    c += (size_t)h->g.nnb * sizeof(int);
    nb.active_list = (int *)c;
    c += (size_t)h->g.nnb * sizeof(int);
    nb.active_n = (int *)c;
    c += 16 * sizeof(int);
    c = (char *)(((uintptr_t)c + 15) & ~(uintptr_t)15);
    if (h->any_node_bc) {
        nb.bc_val = (const float4 *)c;
        CK(h, cudaMemcpyAsync(c, h->nbc_val.data(), (size_t)nn * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
        c += (size_t)nn * sizeof(float4);
        nb.bc_type = (const unsigned char *)c;
        CK(h, cudaMemcpyAsync(c, h->nbc_type.data(), (size_t)nn, cudaMemcpyHostToDevice, h->stream));
        c += (size_t)nn;
        c = (char *)(((uintptr_t)c + 15) & ~(uintptr_t)15);
    }
    if (h->multi) {
        nb.body = (int2 *)c;
        c += (size_t)nn * sizeof(int2);
        nb.has_rigid = (unsigned char *)c;
        c += (size_t)nn;
        c = (char *)(((uintptr_t)c + 15) & ~(uintptr_t)15);
        nb.block_body = (int *)c;
        c += (size_t)ncb * sizeof(int);
        nb.nblk_two = (int *)c;
        c += (size_t)h->g.nnb * sizeof(int);
        // per-(cell, object) smallest particle id + rigid bits
        gy_status st = dalloc(h, &h->d_cell_min, (size_t)h->g.nc * (h->nbody + 1));
        if (st) return st;
        for (int a = 0; a < 3; a++) {
            st = dalloc(h, &h->d_nidx[a], h->nidx[a].size());
            if (st) return st;
            CK(h, cudaMemcpyAsync(h->d_nidx[a], h->nidx[a].data(), h->nidx[a].size() * sizeof(int),
                                  cudaMemcpyHostToDevice, h->stream));
        }
    }
    return GY_OK;
}

// Full conservation sums of the state as set (initialisation, state load): the total mass
// is kept on the host, since steps leave it unchanged and their G2P sums only the rest.
static gy_status sum_state(gy_solver *h)
{
    launch_stats(pview(h, h->cur), h->n, h->d_stats, h->stream);
    double v0 = 0.0;
    CK(h, cudaMemcpyAsync(&v0, h->d_stats, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->mass_total = v0;
    h->stats_fresh = true;
    return GY_OK;
}

gy_status gy_initialize(gy_solver *h, const gy_material *mats, int nmat, const gy_params *prm)
{
    if (!h || !mats || nmat <= 0 || !prm) return GY_ERR_ARG;
    if (h->initialized) return fail(h, GY_ERR_STATE, "already initialized");
    if (nmat > MAX_MATERIALS) return fail(h, GY_ERR_UNSUPPORTED, "more than 4096 materials");
    if ((prm->is3D != 0) != (h->g.is3d != 0))
        return fail(h, GY_ERR_ARG, "Parameters.is3D does not match the grid (L[2] == 0 means 2D)");
    cudaSetDevice(h->device);
    h->mats.assign(mats, mats + nmat);
    h->prm = *prm;
    const long long n = (long long)h->mat.size();
    h->n = n;
    // Solver::Solver dt (Solver.cpp:15-32): maxK seeded with 1, minRho with 1e15
    double maxK = 1.0, minrho = 1e15;
    for (int i = 0; i < nmat; i++) {
        if (mats[i].bulkMod > maxK) maxK = mats[i].bulkMod;
        if (mats[i].density < minrho) minrho = mats[i].density;
    }
    h->dt = prm->CFL * (h->h / std::sqrt(maxK / minrho));
    // object slots, model coverage
    std::map<int, int> slot_of;
    bool any_rigid = false;
    for (long long i = 0; i < n; i++) {
        const int m = h->mat[i];
        if (m < 0 || m >= nmat) return fail(h, GY_ERR_ARG, "particle material id out of range");
        if (slot_of.find(h->obj[i]) == slot_of.end()) {
            const int s = (int)slot_of.size();
            slot_of[h->obj[i]] = s;
        }
        if (mats[m].isRigid) any_rigid = true;
        if (mats[m].model == 3 || mats[m].model == 4 || mats[m].model == 5 || mats[m].isDamage) h->has_dp = true;
    }
    for (long long i = 0; i < n; i++)
        if (h->dmg[i] != 0.0) h->has_dp = true;
    if ((int)slot_of.size() > MAX_BODIES) return fail(h, GY_ERR_UNSUPPORTED, "more than 16 objects");
    h->nbody = std::max(1, (int)slot_of.size());
    h->slot_obj.assign(h->nbody, 0);
    for (auto &kv : slot_of) h->slot_obj[kv.second] = kv.first;
    h->multi = (h->nbody > 1) || any_rigid || h->opt.track_normals;
    for (long long i = 0; i < n; i++)
        if (h->pbc_type[i] >= 33 && h->pbc_type[i] != BC_MP_VX && h->pbc_type[i] != BC_MP_VY &&
            h->pbc_type[i] != BC_MP_VZ && h->pbc_type[i] != BC_MP_VX_VY && h->pbc_type[i] != BC_MP_VXSIN &&
            h->pbc_type[i] != BC_MP_VYSIN && h->pbc_type[i] != BC_MP_SYYSIN && h->pbc_type[i] != BC_MP_FX &&
            h->pbc_type[i] != BC_MP_FY && h->pbc_type[i] != BC_MP_FZ && h->pbc_type[i] != BC_MP_FX_FY &&
            h->pbc_type[i] != BC_MP_STRESS_XX_YY)
            h->pbc_type[i] = 0;  // every other particle BC has no body in the reference

    // ---- particle slab ----
    h->cap = (std::max<long long>(n, 1) + 31) / 32 * 32;  // every field starts on a 128-byte boundary
    const size_t slab_floats = (size_t)PF_COUNT * h->cap;
    for (int s = 0; s < 2; s++) {
        gy_status st = dalloc(h, &h->slab[s], slab_floats);
        if (st) return st;
    }
    std::vector<float> hs(slab_floats, 0.0f);
    std::vector<int> refkey0(h->cap, 0);
    h->key0.assign((size_t)n, 0);
    h->off0.assign((size_t)n * 3, 0.0f);
    std::vector<float4> pbcv(h->cap, make_float4(0.f, 0.f, 0.f, 0.f));
    auto F = [&](int f, long long i) -> float & { return hs[(size_t)f * h->cap + i]; };
    auto I = [&](int f, long long i) -> int & { return reinterpret_cast<int *>(hs.data())[(size_t)f * h->cap + i]; };
    const double hh = h->h, ps2 = h->psep / 2;
    const double init_vol = h->g.is3d ? h->psep * h->psep * h->psep : h->psep * h->psep;
    const int dims_c[3] = {h->g.ncx, h->g.ncy, h->g.ncz};
    for (long long i = 0; i < n; i++) {
        int c[3] = {0, 0, 0};
        for (int a = 0; a < 3; a++) {
            const double x = h->pos[3 * i + a];
            if (a == 2 && !h->g.is3d) {
                F(PF_OZ, i) = 0.0f;
                continue;
            }
            // stencil base as getGIMPNodes computes it (Extrapolation.cpp:658-660)
            int ci = (int)((x - ps2 - 0.0) / hh);
            double off = x / hh - ci;
            // keep the offset in [lp, 1+lp) after rounding
            const double lp = ps2 / hh;
            if (off < lp) { ci -= 1; off += 1.0; }
            if (off >= 1.0 + lp) { ci += 1; off -= 1.0; }
            if (ci < 0 || ci > dims_c[a] - 2)
                return fail(h, GY_ERR_RANGE, "particle " + std::to_string(i) + " lies outside the grid's stencil range");
            c[a] = ci;
            F(PF_OX + a, i) = (float)off;
        }
        I(PF_KEY, i) = encode_key(c[0], c[1], h->g.is3d ? c[2] : 0, h->g);
        h->key0[i] = I(PF_KEY, i);
        for (int a = 0; a < 3; a++) h->off0[3 * i + a] = F(PF_OX + a, i);
        for (int k = 0; k < 3; k++) F(PF_VX + k, i) = (float)h->vel[3 * i + k];
        for (int k = 0; k < 6; k++) F(PF_S0 + k, i) = (float)h->stress[6 * i + k];
        const gy_material &M = mats[h->mat[i]];
        // Solver::initialize (Solver.cpp:40-69)
        const double rho = M.density;
        double mass = rho * init_vol;
        if (h->g.is3d && M.isRigid) mass = 1.0;
        F(PF_RHO, i) = (float)rho;
        F(PF_MASS, i) = (float)mass;
        uint32_t info = (uint32_t)h->mat[i] | ((uint32_t)slot_of[h->obj[i]] << INFO_OBJ_SHIFT) |
                        ((uint32_t)h->pbc_type[i] << INFO_BC_SHIFT) | INFO_INIT_VOL;
        if (h->hold[i]) info |= INFO_HOLD;
        if (M.isRigid) info |= INFO_RIGID;
        I(PF_INFO, i) = (int)info;
        I(PF_PID, i) = (int)i;
        F(PF_DMG, i) = (float)h->dmg[i];
        for (int k = 0; k < 4; k++) (&pbcv[i].x)[k] = (float)h->pbc_val[4 * i + k];
        // the initial binning key has no quarter-cell shift (MaterialPoints.cpp:228-231)
        const int ix = (int)((h->pos[3 * i + 0] - 0.0) / hh), iy = (int)((h->pos[3 * i + 1] - 0.0) / hh),
                  iz = (int)((h->pos[3 * i + 2] - 0.0) / hh);
        refkey0[i] = ix + iy * (h->nx - 1) + iz * (h->nx - 1) * (h->ny - 1);
    }
    CK(h, cudaMemcpyAsync(h->slab[0], hs.data(), slab_floats * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    h->cur = 0;
    gy_status st;
    if ((st = dalloc(h, &h->d_pbc_val, h->cap))) return st;
    CK(h, cudaMemcpyAsync(h->d_pbc_val, pbcv.data(), h->cap * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    if (std::any_of(h->flaw.begin(), h->flaw.end(), [](double w) { return w != 1.0; })) {
        std::vector<float> fw((size_t)h->cap, 1.0f);
        for (long long i = 0; i < h->n; i++) fw[i] = (float)h->flaw[i];
        if ((st = dalloc(h, &h->d_flaw, h->cap))) return st;
        CK(h, cudaMemcpyAsync(h->d_flaw, fw.data(), h->cap * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));  // fw dies on return
    }
    if (h->multi) {
        if ((st = dalloc(h, &h->d_refkey0, h->cap))) return st;
        CK(h, cudaMemcpyAsync(h->d_refkey0, refkey0.data(), h->cap * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    }
    std::vector<DevMaterial> dm(nmat);
    for (int i = 0; i < nmat; i++) dm[i] = to_dev(mats[i]);
    if ((st = dalloc(h, &h->d_mats, nmat))) return st;
    CK(h, cudaMemcpyAsync(h->d_mats, dm.data(), nmat * sizeof(DevMaterial), cudaMemcpyHostToDevice, h->stream));
    if ((st = dalloc(h, &h->d_status, 4))) return st;
    CK(h, cudaMemsetAsync(h->d_status, 0, 4 * sizeof(int), h->stream));
    if ((st = dalloc(h, &h->d_stats, STATS_SLOTS * 8))) return st;
    CK(h, cudaMalloc(&h->d_sc, sizeof(StepScalars)));
    CK(h, cudaMallocHost(&h->h_ring, gy_solver::kRing * sizeof(StepScalars)));
    CK(h, cudaMallocHost(&h->h_rb, sizeof(gy_solver::Readback)));
    for (int k = 0; k < gy_solver::kRing; k++) CK(h, cudaEventCreateWithFlags(&h->ring_ev[k], cudaEventDisableTiming));
    // sort scratch
    h->sort_mem = nullptr;
    const size_t sbytes = sort_scratch_bytes(h->cap);
    CK(h, cudaMalloc(&h->sort_mem, sbytes + 4096));
    {
        int *p = (int *)h->sort_mem;
        const long long nbk = (h->cap + 2047) / 2048;
        h->ws.keys[0] = p; p += h->cap;
        h->ws.keys[1] = p; p += h->cap;
        h->ws.vals[0] = p; p += h->cap;
        h->ws.vals[1] = p; p += h->cap;
        h->ws.hist = p; p += 2 * 256 * nbk;
        h->ws.scan_tmp = p;
        h->ws.cap = h->cap;
        h->ws.nblocks_cap = (int)nbk;
    }
    // incremental re-sort scratch, the two sorted-key buffers and the cell blocks' first
    // positions, zeroed once
    {
        const size_t nblk = (size_t)h->g.nbx * h->g.nby * h->g.nbz;
        const size_t rints = resort_scratch_ints(h->cap) + 2 * (size_t)h->cap + nblk;
        CK(h, cudaMalloc(&h->resort_mem, rints * sizeof(int) + 4096));
        CK(h, cudaMemsetAsync(h->resort_mem, 0, rints * sizeof(int) + 4096, h->stream));
        int *p = (int *)h->resort_mem;
        h->skey_buf[0] = p; p += h->cap;
        h->skey_buf[1] = p; p += h->cap;
        h->d_blk_first = p; p += nblk;
        resort_bind(h->rs, p, h->cap);
        h->sk = 0;
        h->resort_valid = false;
    }
    if ((st = dalloc(h, &h->d_perm, h->cap))) return st;
    // multi-body handles: the second half lists the segments the one-object P2G defers
    if ((st = dalloc(h, &h->d_seg, (h->multi ? 2 : 1) * h->cap))) return st;
    if ((st = dalloc(h, &h->d_nseg, 4))) return st;
    CK(h, cudaMemsetAsync(h->d_nseg, 0, 4 * sizeof(int), h->stream));
    {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        h->persist_grid = sms * p2g_blocks_per_sm();
        h->g2p_grid = sms * g2p_blocks_per_sm(h->has_dp);
    }
    if ((st = alloc_nodes(h))) return st;
    for (long long i = 0; i < n && !h->thermal; i++) h->thermal = h->temp[i] != 0.0;
    if (h->thermal && (st = enable_thermal(h))) return st;
    // the slab goes to the device in insertion order; put it in cell-key order now, so the
    // first step reads it coalesced and re-sorts only the particles that move
    h->resort_valid = false;
    if (n > 0) {
        int key_bits = 1;
        const long long maxkey = (long long)h->g.nbx * h->g.nby * h->g.nbz * 64;
        while ((1LL << key_bits) < maxkey) key_bits++;
        const int *keys = reinterpret_cast<const int *>(h->slab[0]) + (size_t)PF_KEY * h->cap;
        const int *sorted = sort_pairs(keys, h->d_perm, n, key_bits, h->ws, h->stream);
        launch_gather_slab(h->slab[0], h->slab[1], h->d_perm, n, h->cap, PF_COUNT, h->stream);
        if (h->skey_buf[0])
            CK(h, cudaMemcpyAsync(h->skey_buf[0], sorted, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
        h->cur = 1;
        h->sk = 0;
        h->resort_valid = h->skey_buf[0] != nullptr;
    }
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaGetLastError());
    h->initialized = true;
    h->steps = 0;
    h->t_prev = 0.0;
    h->since_sort = 1 << 30;
    h->tables_valid = false;
    return sum_state(h);
}

gy_status gy_set_dt(gy_solver *h, double dt)
{
    if (!h || !(dt > 0)) return GY_ERR_ARG;
    h->dt = dt;
    return GY_OK;
}

gy_status gy_get_dt(const gy_solver *h, double *dt)
{
    if (!h || !dt) return GY_ERR_ARG;
    *dt = h->dt;
    return GY_OK;
}

gy_status gy_set_params(gy_solver *h, const gy_params *prm)
{
    if (!h || !prm) return GY_ERR_ARG;
    if ((prm->is3D != 0) != (h->g.is3d != 0)) return fail(h, GY_ERR_ARG, "is3D does not match the grid");
    h->prm = *prm;
    return GY_OK;
}

gy_status gy_set_options(gy_solver *h, const gy_options *opt)
{
    if (!h || !opt) return GY_ERR_ARG;
    if (opt->sort_every < 1) return fail(h, GY_ERR_ARG, "sort_every must be >= 1");
    if (opt->use_graph != 0 && opt->use_graph != 1) return fail(h, GY_ERR_ARG, "use_graph must be 0 or 1");
    if (opt->p2g_lanes != 3 && opt->p2g_lanes != 9) return fail(h, GY_ERR_ARG, "p2g_lanes must be 3 or 9");
    if (h->initialized && (opt->track_normals != h->opt.track_normals || opt->keep_node_fields != h->opt.keep_node_fields))
        return fail(h, GY_ERR_STATE, "track_normals / keep_node_fields must be set before gy_initialize");
    h->opt = *opt;
    drop_graphs(h);  // captured steps bake the options in
    return GY_OK;
}

gy_status gy_get_options(const gy_solver *h, gy_options *opt)
{
    if (!h || !opt) return GY_ERR_ARG;
    *opt = h->opt;
    return GY_OK;
}

void *gy_stream(gy_solver *h) { return h ? (void *)h->stream : nullptr; }

static StepScalars make_scalars(const gy_solver *h, int step)
{
    StepScalars sc{};
    sc.dt = (float)h->dt;
    sc.dt_node = (float)(step == 1 ? 0.5 * h->dt : h->dt);
    for (int k = 0; k < 3; k++) sc.gravity[k] = (float)h->prm.gravity[k];
    sc.damping = (float)h->prm.damping;
    sc.mu = (float)h->prm.mu;
    sc.t_bc = (float)h->t_prev;
    sc.fixed_grid_bcs = h->prm.fixed_grid_bcs;
    sc.multi_body = h->multi ? 1 : 0;
    sc.init_volume = (float)(h->g.is3d ? h->psep * h->psep * h->psep : h->psep * h->psep);
    sc.step = step;
    return sc;
}

static StepArgs make_args(gy_solver *h)
{
    StepArgs a{};
    a.g = h->g;
    a.sc = h->d_sc;
    a.multi_body = h->multi ? 1 : 0;
    a.mats = h->d_mats;
    a.pbc_val = h->d_pbc_val;
    a.flaw = h->d_flaw;
    // G2P flags the particles that change cell for the next incremental re-sort
    a.mover_mask = h->rs.wmask;
    a.mover_cnt = h->rs.wcnt;
    if (h->dplog_on) {
        a.dp.log_x = h->d_dplog;
        a.dp.log_y = h->d_dplog + (size_t)h->dplog_cap * 16;
        a.dp.log_n = h->d_dplog_n;
        a.dp.log_cap = h->dplog_cap;
        a.dp.log_every = h->dplog_every;
    }
    if (h->surr_on) {
        a.dp.pend = h->d_pend;
        a.dp.pend_n = h->d_pend_n;
        a.dp.pend_cap = (unsigned int)h->n;
    }
    a.status = h->d_status;
    a.stats = h->d_stats;
    return a;
}

// The stream work of one step (no host state changes): sort, P2G, fold + solve, G2P.
static void issue_step(gy_solver *h, const StepVariant &v, cudaEvent_t *tev)
{
    const StepArgs a = make_args(h);
    cudaStream_t s = h->stream;
    if (tev) cudaEventRecord(tev[0], s);
    // (a) stable counting sort of the cell keys; the particle kernels read through perm
    const int *perm = nullptr;
    const int *skey = reinterpret_cast<const int *>(h->slab[v.cur]) + (size_t)PF_KEY * h->cap;
    if (v.sort) {
        int *out = h->skey_buf[v.sk];
        int key_bits = 1;
        const long long maxkey = (long long)h->g.nbx * h->g.nby * h->g.nbz * 64;
        while ((1LL << key_bits) < maxkey) key_bits++;
        if (v.sort == 1) {
            // the slab is in the order of the last sort: re-sort only the particles that moved,
            // which every G2P since that sort has flagged (the mover words start clear, and
            // each re-sort clears them after use)
            resort_keys(skey, h->skey_buf[v.sk ^ 1], out, h->d_perm, h->n, key_bits, h->rs, s, true, h->d_blk_first);
        } else {
            const int *sorted = sort_pairs(skey, h->d_perm, h->n, key_bits, h->ws, s);
            if (h->n > 0 && sorted != out)
                cudaMemcpyAsync(out, sorted, (size_t)h->n * sizeof(int), cudaMemcpyDeviceToDevice, s);
        }
        skey = out;
        perm = h->d_perm;
    }
    // the segment count alternates between two counters by slab parity: this step's block
    // heads fill one and zero the other for the next step, and zero this step's active
    // node-block count and list length
    int *nseg = h->d_nseg + v.cur;
    launch_block_heads(skey, h->n, h->d_seg, nseg, s, h->nb.active_n, h->nb.active_count, h->d_nseg + (v.cur ^ 1),
                       v.sort ? h->d_blk_first : nullptr);
    PView src = pview(h, v.cur), dst = pview(h, v.cur ^ 1);
    // body slots from the sort table of the reference's cadence (Solver.cpp:91)
    if (v.tables) {
        launch_body_tables(src, h->n, a, h->d_cell_min, h->nbody, v.tables == 2 ? h->d_refkey0 : nullptr, s);
        launch_body_assign(h->nb, a, h->d_cell_min, h->nbody, h->d_nidx[0], h->d_nidx[1], h->d_nidx[2], s);
    }
    if (tev) cudaEventRecord(tev[1], s);
    // (b) P2G
    // heat conduction: fused into the single-body P2G, a separate pass for body slots
    const bool fused_thermal = h->thermal && !h->multi;
    // multi-body: the one-object segments take the plane-lane kernel unless normals are tracked
    int *defer = nullptr, *ndefer = nullptr;
    if (h->multi && !h->opt.track_normals) {
        defer = h->d_seg + h->cap;
        ndefer = h->d_nseg + 2;
        cudaMemsetAsync(ndefer, 0, sizeof(int), s);
    }
    launch_p2g(src, perm, skey, h->n, h->d_seg, nseg, h->persist_grid, h->nb, a, s,
               fused_thermal ? h->d_therm : nullptr, fused_thermal ? h->d_tnode : nullptr, h->opt.p2g_lanes, defer,
               ndefer);
    if (h->thermal && h->multi)
        launch_thermal_p2g(src, h->d_therm, perm, skey, h->n, h->d_seg, nseg, h->d_tnode, a, s);
    if (tev) cudaEventRecord(tev[2], s);
    // (c) periodic fold, nodal solve, grid BCs
    launch_fold(h->nb, a, s);
    launch_solve(h->nb, a, h->opt.keep_node_fields != 0, s);
    if (tev) cudaEventRecord(tev[3], s);
    // (d) G2P + particle BCs + update + constitutive + damage, written in sorted order, with
    // the conservation sums of the updated state (their partials zeroed by the compaction)
    if (h->surr_on) cudaMemsetAsync(h->d_pend_n, 0, sizeof(unsigned int), s);
    launch_g2p_update(src, dst, perm, skey, h->n, h->d_seg, nseg, h->g2p_grid, h->nb, a,
                      h->opt.track_normals != 0, h->opt.check_finite != 0, h->has_dp, s,
                      fused_thermal ? h->d_therm : nullptr, fused_thermal ? h->d_tnode : nullptr);
    if (h->surr_on)
        launch_dp_surrogate(dst, h->d_pend, h->d_pend_n, (unsigned int)h->n, h->d_mats, h->d_surr, h->d_sc, h->d_flaw,
                            h->surr_tol, h->d_surr_counts, h->d_status, s);
    if (h->thermal && h->multi)
        launch_thermal_g2p(src, h->d_therm, perm, skey, h->n, h->d_seg, nseg, h->d_tnode, h->nb, a, s);
    else if (h->thermal)
        launch_thermal_clear(h->nb, a, h->d_tnode, s);
    if (tev) cudaEventRecord(tev[4], s);
}

static gy_status enqueue_step(gy_solver *h, double t, int step)
{
    cudaStream_t s = h->stream;
    h->stats_fresh = false;
    const bool timing = h->phase_timing && h->tev_used < kMaxTimedSteps;
    cudaEvent_t *tev = nullptr;
    if (timing) {
        const size_t need = (size_t)(h->tev_used + 1) * 5;
        while (h->tev.size() < need) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            h->tev.push_back(e);
        }
        tev = &h->tev[(size_t)h->tev_used * 5];
        h->tev_used++;
    }
    // host decisions for this step
    StepVariant v{h->cur, h->sk, 0, 0};
    if (h->since_sort >= h->opt.sort_every) {
        v.sort = (h->resort_valid && !h->opt.full_sort) ? 1 : 2;
        v.sk = h->sk ^ 1;
    }
    if (h->multi && ((step % 10 == 0) || step == 1 || !h->tables_valid)) v.tables = h->steps == 0 ? 2 : 1;
    // every step's scalars (dt, dt at the nodes, gravity, damping, friction, BC time) travel
    // host-to-device through a pinned ring slot, ahead of the step's kernels on its stream; a
    // slot is rewritten only after the copy that last read it has run (the host waits only
    // when 32 steps are queued)
    {
        const int slot = (int)(h->ring_pos++ % gy_solver::kRing);
        if (h->ring_busy[slot]) CK(h, cudaEventSynchronize(h->ring_ev[slot]));
        h->h_ring[slot] = make_scalars(h, step);
        CK(h, cudaMemcpyAsync(h->d_sc, &h->h_ring[slot], sizeof(StepScalars), cudaMemcpyHostToDevice, s));
        CK(h, cudaEventRecord(h->ring_ev[slot], s));
        h->ring_busy[slot] = true;
    }
    if (h->opt.use_graph && !timing) {
        StepGraph *gr = nullptr;
        for (auto &c : h->graphs)
            if (c.v == v) gr = &c;
        if (!gr) {
            if (h->graphs.size() >= 8) drop_graphs(h);
            StepGraph ng{};
            ng.v = v;
            const long long l0 = launch_count();
            CK(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            issue_step(h, v, nullptr);
            cudaGraph_t graph = nullptr;
            CK(h, cudaStreamEndCapture(s, &graph));
            ng.launches = launch_count() - l0;
            const cudaError_t ei = cudaGraphInstantiate(&ng.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ei != cudaSuccess) return fail(h, GY_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
            note_launch(-(int)ng.launches);  // counted again per replay below
            h->graphs.push_back(ng);
            gr = &h->graphs.back();
        }
        CK(h, cudaGraphLaunch(gr->exec, s));
        note_launch((int)gr->launches);
    } else {
        issue_step(h, v, tev);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(h, GY_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    // host bookkeeping
    if (v.sort) {
        h->sk = v.sk;
        h->since_sort = 0;
        h->resort_valid = true;  // this step's G2P writes the slab in this order
    }
    h->since_sort++;
    if (v.tables) h->tables_valid = true;
    h->cur ^= 1;
    h->t_prev = t;
    h->steps++;
    h->stats_fresh = true;
    return GY_OK;
}

gy_status gy_step(gy_solver *h, double t, int step)
{
    if (!h) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "gy_step before gy_initialize");
    cudaSetDevice(h->device);
    if (h->nb.active_count == nullptr) h->nb.active_count = h->d_status + 2;
    return enqueue_step(h, t, step);
}

gy_status gy_steps(gy_solver *h, double t0, int step0, int nsteps, int use_graph)
{
    if (!h || nsteps < 0 || use_graph < 0 || use_graph > 1) return GY_ERR_ARG;
    const int keep = h->opt.use_graph;
    h->opt.use_graph = use_graph;
    gy_status st = GY_OK;
    for (int k = 0; k < nsteps && st == GY_OK; k++) st = gy_step(h, t0 + k * h->dt, step0 + k);
    h->opt.use_graph = keep;
    return st;
}

gy_status gy_sync(gy_solver *h)
{
    if (!h) return GY_ERR_ARG;
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    if (!h->initialized) return GY_OK;
    int flags[4] = {0, 0, 0, 0};
    CK(h, cudaMemcpy(flags, h->d_status, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[0]) {
        CK(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        if (flags[0] & ERR_TC_TIMEOUT) return fail(h, GY_ERR_CUDA, "a tensor-core wait gave up");
        if (flags[0] & ERR_NONFINITE) return fail(h, GY_ERR_NONFINITE, "NaN or Inf in particle state");
        return fail(h, GY_ERR_RANGE, "a particle left the grid's stencil range (clamped)");
    }
    return GY_OK;
}

gy_status gy_num_particles(const gy_solver *h, int64_t *n)
{
    if (!h || !n) return GY_ERR_ARG;
    *n = (int64_t)h->mat.size();
    return GY_OK;
}

static gy_status fetch_slab(gy_solver *h, std::vector<float> &hs)
{
    cudaSetDevice(h->device);
    hs.resize((size_t)PF_COUNT * h->cap);
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(hs.data(), h->slab[h->cur], hs.size() * sizeof(float), cudaMemcpyDeviceToHost));
    return GY_OK;
}

static const int kPWidth[GY_P_NFIELDS] = {3, 3, 3, 3, 6, 6, 6, 1, 1, 1, 1, 1, 1, 3, 1, 3};

gy_status gy_get_particles(gy_solver *h, int field, double *out, int64_t count)
{
    if (!h || !out || field < 0 || field >= GY_P_NFIELDS) return GY_ERR_ARG;
    const int w = kPWidth[field];
    const long long n = (long long)h->mat.size();
    if (count != (int64_t)n * w) return fail(h, GY_ERR_ARG, "count must be n * width");
    if (!h->initialized) {
        // before the solver exists the host staging is authoritative
        for (long long i = 0; i < n; i++) {
            for (int k = 0; k < w; k++) {
                double v = 0.0;
                switch (field) {
                case GY_P_POS: case GY_P_POS0: v = h->pos[3 * i + k]; break;
                case GY_P_VEL: v = h->vel[3 * i + k]; break;
                case GY_P_STRESS: v = h->stress[6 * i + k]; break;
                case GY_P_DAMAGE: v = h->dmg[i]; break;
                case GY_P_TEMP: v = h->temp[i]; break;
                default: v = 0.0;
                }
                out[(size_t)i * w + k] = v;
            }
        }
        return GY_OK;
    }
    if (field == GY_P_TEMP || field == GY_P_TEMPGRAD) {
        // kept by insertion index; without a device copy every temperature is the host value
        // and every gradient zero
        std::vector<float4> th;
        if (h->d_therm) {
            th.resize((size_t)n);
            cudaSetDevice(h->device);
            CK(h, cudaStreamSynchronize(h->stream));
            CK(h, cudaMemcpy(th.data(), h->d_therm, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
        }
        for (long long i = 0; i < n; i++) {
            if (field == GY_P_TEMP) {
                out[i] = h->d_therm ? (double)th[i].x : h->temp[i];
            } else {
                out[3 * i] = h->d_therm ? (double)th[i].y : 0.0;
                out[3 * i + 1] = h->d_therm ? (double)th[i].z : 0.0;
                out[3 * i + 2] = h->d_therm ? (double)th[i].w : 0.0;
            }
        }
        return GY_OK;
    }
    std::vector<float> hs;
    gy_status st = fetch_slab(h, hs);
    if (st) return st;
    auto F = [&](int f, long long i) { return hs[(size_t)f * h->cap + i]; };
    auto I = [&](int f, long long i) { return reinterpret_cast<const int *>(hs.data())[(size_t)f * h->cap + i]; };
    const double hh = h->h;
    for (long long i = 0; i < n; i++) {
        const long long pid = I(PF_PID, i);
        double *o = out + (size_t)pid * w;
        const uint32_t info = (uint32_t)I(PF_INFO, i);
        switch (field) {
        case GY_P_POS:
        case GY_P_DISP: {
            // displacement from the change of (cell, FP32 offset) since upload, so that a
            // particle that has not moved reports exactly zero; position = pos0 + disp
            int c[3], c0[3];
            auto split = [&](int key, int *cc) { decode_key(key, h->g, cc[0], cc[1], cc[2]); };
            split(I(PF_KEY, i), c);
            split(h->key0[pid], c0);
            for (int k = 0; k < 3; k++) {
                double d = 0.0;
                if (k < 2 || h->g.is3d)
                    d = ((double)(c[k] - c0[k]) + ((double)F(PF_OX + k, i) - (double)h->off0[3 * pid + k])) * hh;
                o[k] = field == GY_P_POS ? h->pos[3 * pid + k] + d : d;
            }
            break;
        }
        case GY_P_POS0: for (int k = 0; k < 3; k++) o[k] = h->pos[3 * pid + k]; break;
        case GY_P_VEL: for (int k = 0; k < 3; k++) o[k] = F(PF_VX + k, i); break;
        case GY_P_STRESS: for (int k = 0; k < 6; k++) o[k] = F(PF_S0 + k, i); break;
        case GY_P_STRAIN: for (int k = 0; k < 6; k++) o[k] = F(PF_E0 + k, i); break;
        case GY_P_PSTRAIN: for (int k = 0; k < 6; k++) o[k] = h->has_dp ? F(PF_EP0 + k, i) : 0.0; break;
        case GY_P_EQPS: o[0] = h->has_dp ? F(PF_EQPS, i) : 0.0; break;
        case GY_P_DAMAGE: o[0] = h->has_dp ? F(PF_DMG, i) : 0.0; break;
        case GY_P_SMAX: o[0] = h->has_dp ? F(PF_SMAX, i) : 0.0; break;
        case GY_P_MASS: o[0] = F(PF_MASS, i); break;
        case GY_P_DENSITY: o[0] = F(PF_RHO, i); break;
        case GY_P_VOLUME:
            o[0] = (info & INFO_INIT_VOL) ? (h->g.is3d ? h->psep * h->psep * h->psep : h->psep * h->psep)
                                          : (double)F(PF_MASS, i) / (double)F(PF_RHO, i);
            break;
        case GY_P_NORMALS: for (int k = 0; k < 3; k++) o[k] = h->opt.track_normals ? F(PF_NX + k, i) : 0.0; break;
        default: break;
        }
    }
    return GY_OK;
}

gy_status gy_get_particles_int(gy_solver *h, int field, int *out, int64_t count)
{
    if (!h || !out) return GY_ERR_ARG;
    const long long n = (long long)h->mat.size();
    if (count != (int64_t)n) return fail(h, GY_ERR_ARG, "count must be n");
    if (!h->initialized) {
        for (long long i = 0; i < n; i++) {
            if (field == GY_PI_MATERIAL) out[i] = h->mat[i];
            else if (field == GY_PI_OBJECT) out[i] = h->obj[i];
            else if (field == GY_PI_DEVICE_SLOT) out[i] = (int)i;
            else if (field == GY_PI_CELLID) {
                const int ix = (int)(h->pos[3 * i] / h->h), iy = (int)(h->pos[3 * i + 1] / h->h),
                          iz = (int)(h->pos[3 * i + 2] / h->h);
                out[i] = ix + iy * (h->nx - 1) + iz * (h->nx - 1) * (h->ny - 1);
            } else return GY_ERR_ARG;
        }
        return GY_OK;
    }
    std::vector<float> hs;
    gy_status st = fetch_slab(h, hs);
    if (st) return st;
    auto F = [&](int f, long long i) { return hs[(size_t)f * h->cap + i]; };
    auto I = [&](int f, long long i) { return reinterpret_cast<const int *>(hs.data())[(size_t)f * h->cap + i]; };
    for (long long i = 0; i < n; i++) {
        const long long pid = I(PF_PID, i);
        const uint32_t info = (uint32_t)I(PF_INFO, i);
        switch (field) {
        case GY_PI_MATERIAL: out[pid] = info_mat(info); break;
        case GY_PI_OBJECT: out[pid] = h->slot_obj[info_obj(info)]; break;
        case GY_PI_DEVICE_SLOT: out[pid] = (int)i; break;
        case GY_PI_CELLID: {
            if (info & INFO_INIT_VOL) {
                // no update yet: the initial unshifted key (MaterialPoints.cpp:228-231)
                const int ix = (int)(h->pos[3 * pid] / h->h), iy = (int)(h->pos[3 * pid + 1] / h->h),
                          iz = (int)(h->pos[3 * pid + 2] / h->h);
                out[pid] = ix + iy * (h->nx - 1) + iz * (h->nx - 1) * (h->ny - 1);
                break;
            }
            int c[3];
            decode_key(I(PF_KEY, i), h->g, c[0], c[1], c[2]);
            int id[3] = {0, 0, 0};
            for (int k = 0; k < (h->g.is3d ? 3 : 2); k++) id[k] = (int)((c[k] + (double)F(PF_OX + k, i)) - 0.25);
            out[pid] = id[0] + id[1] * (h->nx - 1) + id[2] * (h->nx - 1) * (h->ny - 1);
            break;
        }
        default: return GY_ERR_ARG;
        }
    }
    return GY_OK;
}

gy_status gy_get_nodes(gy_solver *h, int field, double *out, int64_t count)
{
    if (!h || !out || field < 0 || field >= GY_N_NFIELDS) return GY_ERR_ARG;
    const int w = field == GY_N_MASS ? 1 : 3;
    if (count != (int64_t)h->nn * w) return fail(h, GY_ERR_ARG, "count must be numNodes * width");
    if (!h->initialized) {
        std::fill(out, out + count, 0.0);
        return GY_OK;
    }
    if ((field == GY_N_VEL || field == GY_N_FORCE) && !h->opt.keep_node_fields)
        return fail(h, GY_ERR_STATE, "node velocity/force need gy_options.keep_node_fields = 1");
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    std::vector<float4> buf((size_t)h->nn);
    const float4 *src = field == GY_N_MASS || field == GY_N_VEL1 ? h->nb.gv
                        : field == GY_N_ACC1                     ? h->nb.ga
                        : field == GY_N_VEL                      ? h->nb.out_com
                                                                 : h->nb.out_force;
    CK(h, cudaMemcpy(buf.data(), src, (size_t)h->nn * sizeof(float4), cudaMemcpyDeviceToHost));
    for (long long i = 0; i < h->nn; i++) {
        const float4 v = buf[i];
        if (field == GY_N_MASS) out[i] = v.x;
        else if (field == GY_N_VEL1) { out[3 * i] = v.y; out[3 * i + 1] = v.z; out[3 * i + 2] = v.w; }
        else { out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z; }
    }
    return GY_OK;
}

gy_status gy_get_stats(gy_solver *h, gy_stats *out)
{
    if (!h || !out) return GY_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    if (!h->initialized) return GY_OK;
    cudaSetDevice(h->device);
    // the last step's G2P summed the state it wrote (all but the mass, which is summed when
    // the state is set); otherwise sum it here
    if (!h->stats_fresh) {
        gy_status st = sum_state(h);
        if (st) return st;
    }
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double *part = h->h_rb->part;
    const int *flags = h->h_rb->flags;
    CK(h, cudaMemcpyAsync(h->h_rb->part, h->d_stats, sizeof(h->h_rb->part), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(h->h_rb->flags, h->d_status, sizeof(h->h_rb->flags), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int q = 0; q < STATS_SLOTS; q++)
        for (int k = 1; k < 8; k++) v[k] += part[q * 8 + k];
    v[0] = h->mass_total;
    out->mass = v[0];
    out->momentum[0] = v[1];
    out->momentum[1] = v[2];
    out->momentum[2] = v[3];
    out->kinetic = v[4];
    out->strain_energy = v[5];
    out->active_nodes = flags[2];
    out->steps = h->steps;
    out->status_flags = flags[0];
    return GY_OK;
}

gy_status gy_set_phase_timing(gy_solver *h, int on)
{
    if (!h) return GY_ERR_ARG;
    h->phase_timing = on != 0;
    h->tev_used = 0;
    return GY_OK;
}

gy_status gy_get_phase_times(gy_solver *h, float *ms5, int64_t *steps)
{
    if (!h || !ms5) return GY_ERR_ARG;
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 5; k++) ms5[k] = 0.f;
    for (long long q = 0; q < h->tev_used; q++) {
        cudaEvent_t *e = &h->tev[(size_t)q * 5];
        for (int k = 0; k < 4; k++) {
            float ms = 0.f;
            CK(h, cudaEventElapsedTime(&ms, e[k], e[k + 1]));
            ms5[k] += ms;
        }
        float tot = 0.f;
        CK(h, cudaEventElapsedTime(&tot, e[0], e[4]));
        ms5[4] += tot;
    }
    if (steps) *steps = h->tev_used;
    h->tev_used = 0;
    return GY_OK;
}

gy_status gy_time_steps(gy_solver *h, double t0, int step0, int nsteps, float *ms)
{
    if (!h || !ms || nsteps < 0) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "gy_time_steps before gy_initialize");
    cudaSetDevice(h->device);
    CK(h, cudaEventRecord(h->ev[0], h->stream));
    gy_status st = gy_steps(h, t0, step0, nsteps, 0);
    if (st) return st;
    CK(h, cudaEventRecord(h->ev[5], h->stream));
    CK(h, cudaEventSynchronize(h->ev[5]));
    CK(h, cudaEventElapsedTime(ms, h->ev[0], h->ev[5]));
    return GY_OK;
}

int64_t gy_kernel_launches(void) { return (int64_t)launch_count(); }

// ---- checkpoint / resume ----
namespace {
struct StateHeader {
    char magic[8];            // "GYSTATE1"
    int64_t n, cap, nn, nc;
    int32_t nbody, multi, has_dp, track_normals;
    int64_t steps;
    double t_prev, dt;
    int32_t tables_valid, thermal;
};

size_t state_table_ints(const gy_solver *h) { return h->multi ? (size_t)h->g.nc * (h->nbody + 1) : 0; }
size_t state_bytes(const gy_solver *h, bool thermal)
{
    return sizeof(StateHeader) + (size_t)PF_COUNT * h->n * sizeof(float) + state_table_ints(h) * sizeof(int) +
           (h->multi ? (size_t)h->nn * (sizeof(int2) + 1) : 0) + (thermal ? (size_t)h->n * sizeof(float4) : 0);
}
}  // namespace

gy_status gy_state_size(const gy_solver *h, int64_t *bytes)
{
    if (!h || !bytes) return GY_ERR_ARG;
    if (!h->initialized) return GY_ERR_STATE;
    *bytes = (int64_t)state_bytes(h, h->d_therm != nullptr);
    return GY_OK;
}

gy_status gy_state_save(gy_solver *h, void *buf, int64_t bytes)
{
    if (!h || !buf) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "nothing to save before gy_initialize");
    if (bytes < (int64_t)state_bytes(h, h->d_therm != nullptr))
        return fail(h, GY_ERR_ARG, "buffer smaller than gy_state_size");
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    StateHeader hd{};
    std::memcpy(hd.magic, "GYSTATE1", 8);
    hd.n = h->n; hd.cap = h->cap; hd.nn = h->nn; hd.nc = h->g.nc;
    hd.nbody = h->nbody; hd.multi = h->multi; hd.has_dp = h->has_dp; hd.track_normals = h->opt.track_normals;
    hd.steps = h->steps; hd.t_prev = h->t_prev; hd.dt = h->dt; hd.tables_valid = h->tables_valid;
    hd.thermal = h->d_therm ? 1 : 0;
    char *p = static_cast<char *>(buf);
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    for (int f = 0; f < PF_COUNT; f++) {
        CK(h, cudaMemcpy(p, h->slab[h->cur] + (size_t)f * h->cap, (size_t)h->n * sizeof(float), cudaMemcpyDeviceToHost));
        p += (size_t)h->n * sizeof(float);
    }
    if (h->multi) {
        CK(h, cudaMemcpy(p, h->d_cell_min, state_table_ints(h) * sizeof(int), cudaMemcpyDeviceToHost));
        p += state_table_ints(h) * sizeof(int);
        CK(h, cudaMemcpy(p, h->nb.body, (size_t)h->nn * sizeof(int2), cudaMemcpyDeviceToHost));
        p += (size_t)h->nn * sizeof(int2);
        CK(h, cudaMemcpy(p, h->nb.has_rigid, (size_t)h->nn, cudaMemcpyDeviceToHost));
        p += (size_t)h->nn;
    }
    if (h->d_therm) CK(h, cudaMemcpy(p, h->d_therm, (size_t)h->n * sizeof(float4), cudaMemcpyDeviceToHost));
    return GY_OK;
}

gy_status gy_state_load(gy_solver *h, const void *buf, int64_t bytes)
{
    if (!h || !buf) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "gy_state_load needs a handle built with gy_initialize");
    if (bytes < (int64_t)sizeof(StateHeader)) return fail(h, GY_ERR_ARG, "buffer too small");
    StateHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    if (std::memcmp(hd.magic, "GYSTATE1", 8) != 0) return fail(h, GY_ERR_ARG, "not a graphyt GPU state");
    if (hd.n != h->n || hd.nn != h->nn || hd.nc != h->g.nc || hd.nbody != h->nbody || hd.multi != (int)h->multi ||
        hd.has_dp != (int)h->has_dp || hd.track_normals != h->opt.track_normals)
        return fail(h, GY_ERR_ARG, "state belongs to a different model (grid, particles, bodies or options differ)");
    if (bytes < (int64_t)state_bytes(h, hd.thermal != 0)) return fail(h, GY_ERR_ARG, "buffer shorter than the state");
    // a handle that carries temperatures cannot take a state saved without them: it would
    // keep its own temperatures and step on differently from the run that was saved
    if (!hd.thermal && h->d_therm)
        return fail(h, GY_ERR_ARG, "state saved without heat conduction, this handle has temperatures");
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    const char *p = static_cast<const char *>(buf) + sizeof(hd);
    for (int f = 0; f < PF_COUNT; f++) {
        CK(h, cudaMemcpy(h->slab[h->cur] + (size_t)f * h->cap, p, (size_t)h->n * sizeof(float), cudaMemcpyHostToDevice));
        p += (size_t)h->n * sizeof(float);
    }
    if (h->multi) {
        CK(h, cudaMemcpy(h->d_cell_min, p, state_table_ints(h) * sizeof(int), cudaMemcpyHostToDevice));
        p += state_table_ints(h) * sizeof(int);
        CK(h, cudaMemcpy(h->nb.body, p, (size_t)h->nn * sizeof(int2), cudaMemcpyHostToDevice));
        p += (size_t)h->nn * sizeof(int2);
        CK(h, cudaMemcpy(h->nb.has_rigid, p, (size_t)h->nn, cudaMemcpyHostToDevice));
        launch_block_body(h->nb, h->g, h->stream);
        p += (size_t)h->nn;
    }
    if (hd.thermal) {
        gy_status st = enable_thermal(h);
        if (st) return st;
        CK(h, cudaMemcpy(h->d_therm, p, (size_t)h->n * sizeof(float4), cudaMemcpyHostToDevice));
        CK(h, cudaMemset(h->d_tnode, 0, (size_t)h->nn * sizeof(float2)));
        if (!h->thermal) {
            h->thermal = true;
            drop_graphs(h);
        }
    }
    h->steps = hd.steps;
    h->t_prev = hd.t_prev;
    h->dt = hd.dt;
    h->tables_valid = hd.tables_valid != 0;
    h->since_sort = 1 << 30;
    h->resort_valid = false;
    return sum_state(h);
}

gy_status gy_sort_keys(const int *keys, int64_t n, int *perm_out, int device)
{
    if (n < 0 || (n > 0 && (!keys || !perm_out))) return GY_ERR_ARG;
    if (n == 0) return GY_OK;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return GY_ERR_CUDA;
    int maxk = 0;
    for (int64_t i = 0; i < n; i++) {
        if (keys[i] < 0) return GY_ERR_ARG;
        maxk = std::max(maxk, keys[i]);
    }
    int bits = 1;
    while ((1LL << bits) <= maxk) bits++;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GY_ERR_CUDA;
    int *d_in = nullptr, *d_perm = nullptr, *mem = nullptr;
    gy_status st = GY_OK;
    const long long nbk = (n + 2047) / 2048;
    if (cudaMalloc(&d_in, n * sizeof(int)) != cudaSuccess || cudaMalloc(&d_perm, n * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&mem, sort_scratch_bytes(n) + 4096) != cudaSuccess) {
        st = GY_ERR_NOMEM;
    } else {
        SortScratch ws{};
        int *p = mem;
        ws.keys[0] = p; p += n;
        ws.keys[1] = p; p += n;
        ws.vals[0] = p; p += n;
        ws.vals[1] = p; p += n;
        ws.hist = p; p += 2 * 256 * nbk;
        ws.scan_tmp = p;
        ws.cap = n;
        ws.nblocks_cap = (int)nbk;
        cudaMemcpyAsync(d_in, keys, n * sizeof(int), cudaMemcpyHostToDevice, s);
        (void)sort_pairs(d_in, d_perm, n, bits, ws, s);
        cudaMemcpyAsync(perm_out, d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) st = GY_ERR_CUDA;
    }
    if (d_in) cudaFree(d_in);
    if (d_perm) cudaFree(d_perm);
    if (mem) cudaFree(mem);
    cudaStreamDestroy(s);
    return st;
}


gy_status gy_resort_keys(const int *keys, const int *prev_sorted, int64_t n, int *perm_out, int *sorted_out,
                         int device)
{
    if (n < 0 || (n > 0 && (!keys || !prev_sorted || !perm_out || !sorted_out))) return GY_ERR_ARG;
    if (n == 0) return GY_OK;
    if (n >= (1LL << 31) - 2) return GY_ERR_ARG;
    int maxk = 0;
    for (int64_t i = 0; i < n; i++) {
        if (keys[i] < 0 || prev_sorted[i] < 0) return GY_ERR_ARG;
        if (i > 0 && prev_sorted[i] < prev_sorted[i - 1]) return GY_ERR_ARG;
        maxk = std::max(maxk, keys[i]);
    }
    int bits = 1;
    while ((1LL << bits) <= maxk) bits++;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return GY_ERR_CUDA;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GY_ERR_CUDA;
    int *mem = nullptr;
    gy_status st = GY_OK;
    const size_t rints = resort_scratch_ints(n) + 4 * (size_t)n;
    if (cudaMalloc(&mem, rints * sizeof(int) + 4096) != cudaSuccess) {
        st = GY_ERR_NOMEM;
    } else {
        int *d_key = mem, *d_prev = mem + n, *d_perm = mem + 2 * n, *d_sorted = mem + 3 * n;
        ResortScratch rs{};
        cudaMemsetAsync(mem + 4 * n, 0, (rints - 4 * (size_t)n) * sizeof(int) + 4096, s);
        resort_bind(rs, mem + 4 * n, n);
        cudaMemcpyAsync(d_key, keys, n * sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_prev, prev_sorted, n * sizeof(int), cudaMemcpyHostToDevice, s);
        resort_keys(d_key, d_prev, d_sorted, d_perm, n, bits, rs, s);
        cudaMemcpyAsync(perm_out, d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(sorted_out, d_sorted, n * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) st = GY_ERR_CUDA;
    }
    if (mem) cudaFree(mem);
    cudaStreamDestroy(s);
    return st;
}

}  // extern "C"

// ---- learned Drucker-Prager surrogate ----------------------------------------------------

extern "C" int64_t gy_mlp_param_count(void);
extern "C" gy_status gy_mlp_train(float *d_params, const float *d_X, const float *d_T, int64_t n, int steps, int batch,
                                  float lr, uint64_t seed, int init, float *loss_out, int *d_status, void *stream);

gy_status gy_dp_log_begin(gy_solver *h, int64_t cap, int every)
{
    if (!h || cap < 1 || cap > 0x7fffffff || every < 1) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "gy_dp_log_begin needs an initialized solver");
    cudaSetDevice(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->d_dplog && h->dplog_cap != (unsigned int)cap) {
        cudaFree(h->d_dplog);
        h->d_dplog = nullptr;
    }
    gy_status st;
    if (!h->d_dplog && (st = dalloc(h, &h->d_dplog, (size_t)cap * (16 + 7)))) return st;
    if (!h->d_dplog_n && (st = dalloc(h, &h->d_dplog_n, 1))) return st;
    CK(h, cudaMemsetAsync(h->d_dplog_n, 0, sizeof(unsigned int), h->stream));
    h->dplog_cap = (unsigned int)cap;
    h->dplog_every = every;
    h->dplog_on = true;
    drop_graphs(h);
    return GY_OK;
}

gy_status gy_dp_log_end(gy_solver *h)
{
    if (!h) return GY_ERR_ARG;
    if (h->dplog_on) {
        h->dplog_on = false;
        drop_graphs(h);
    }
    return GY_OK;
}

static gy_status dplog_count(gy_solver *h, unsigned int *out)
{
    unsigned int c = 0;
    if (h->d_dplog_n) {
        CK(h, cudaMemcpyAsync(&c, h->d_dplog_n, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    *out = std::min(c, h->dplog_cap);
    return GY_OK;
}

gy_status gy_dp_log_count(gy_solver *h, int64_t *count)
{
    if (!h || !count) return GY_ERR_ARG;
    unsigned int c = 0;
    gy_status st = dplog_count(h, &c);
    *count = c;
    return st;
}

gy_status gy_dp_log_read(gy_solver *h, float *x16, float *y7, int64_t max_records)
{
    if (!h || !x16 || !y7 || max_records < 0) return GY_ERR_ARG;
    unsigned int c = 0;
    gy_status st = dplog_count(h, &c);
    if (st) return st;
    const size_t m = (size_t)std::min<int64_t>(c, max_records);
    if (m == 0) return GY_OK;
    CK(h, cudaMemcpyAsync(x16, h->d_dplog, m * 16 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(y7, h->d_dplog + (size_t)h->dplog_cap * 16, m * 7 * sizeof(float), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return GY_OK;
}

static gy_status surr_alloc(gy_solver *h)
{
    gy_status st;
    if (!h->d_surr && (st = dalloc(h, &h->d_surr, (size_t)gy_mlp_param_count()))) return st;
    if (!h->d_surr_counts) {
        if ((st = dalloc(h, &h->d_surr_counts, 2))) return st;
        CK(h, cudaMemsetAsync(h->d_surr_counts, 0, 2 * sizeof(unsigned long long), h->stream));
    }
    return GY_OK;
}

gy_status gy_dp_surrogate_train(gy_solver *h, int steps, int batch, float lr, uint64_t seed, float *loss_out)
{
    if (!h || steps < 0 || batch < 128 || batch % 128 || !(lr > 0.f)) return GY_ERR_ARG;
    cudaSetDevice(h->device);
    unsigned int c = 0;
    gy_status st = dplog_count(h, &c);
    if (st) return st;
    if (c == 0) return fail(h, GY_ERR_STATE, "no logged Drucker-Prager returns to train on (gy_dp_log_begin)");
    if ((st = surr_alloc(h))) return st;
    const float *X = h->d_dplog, *T = h->d_dplog + (size_t)h->dplog_cap * 16;
    st = gy_mlp_train(h->d_surr, X, T, c, steps, batch, lr, seed, 1, loss_out, h->d_status, h->stream);
    if (st) return fail(h, st, "surrogate training failed");
    return GY_OK;
}

gy_status gy_set_dp_surrogate(gy_solver *h, const float *params, int on, float tol)
{
    if (!h || !(tol > 0.f)) return GY_ERR_ARG;
    if (!h->initialized) return fail(h, GY_ERR_STATE, "gy_set_dp_surrogate needs an initialized solver");
    cudaSetDevice(h->device);
    gy_status st;
    if ((st = surr_alloc(h))) return st;
    if (params) {
        CK(h, cudaMemcpyAsync(h->d_surr, params, (size_t)gy_mlp_param_count() * sizeof(float), cudaMemcpyHostToDevice,
                              h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    if (on && !h->d_pend) {
        if ((st = dalloc(h, &h->d_pend, (size_t)h->cap * 2))) return st;
        if ((st = dalloc(h, &h->d_pend_n, 1))) return st;
        CK(h, cudaMemsetAsync(h->d_pend_n, 0, sizeof(unsigned int), h->stream));
    }
    h->surr_tol = tol;
    if ((on != 0) != h->surr_on) {
        h->surr_on = on != 0;
        drop_graphs(h);
    }
    return GY_OK;
}

gy_status gy_get_dp_surrogate(gy_solver *h, float *params)
{
    if (!h || !params) return GY_ERR_ARG;
    if (!h->d_surr) return fail(h, GY_ERR_STATE, "no surrogate parameters");
    CK(h, cudaMemcpyAsync(params, h->d_surr, (size_t)gy_mlp_param_count() * sizeof(float), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return GY_OK;
}

gy_status gy_dp_surrogate_counts(gy_solver *h, int64_t *kept, int64_t *fallback)
{
    if (!h || !kept || !fallback) return GY_ERR_ARG;
    unsigned long long c[2] = {0, 0};
    if (h->d_surr_counts) {
        CK(h, cudaMemcpyAsync(c, h->d_surr_counts, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    *kept = (int64_t)c[0];
    *fallback = (int64_t)c[1];
    return GY_OK;
}
