// mbg_batch.cu -- batched independent periodic domains in the 16-bit form.
//
// The reference runs one domain per process.  Here many small periodic
// domains advance together: each domain is one padded box of a single
// storage array, with its own size, physical extent (per-axis 1/dx for the
// q-correction gradient), viscosity and diffusivity.  A step is
//   k_halo_periodic16 : every box's pad from the opposite faces of that box
//   step variant      : two-pass (Q_corr pass + collision pass) or the fused
//                       step over a work list of column tiles, run by a
//                       persistent grid of (resident CTAs per SM) x (SMs)
// for all domains at once.  Two steps (there and back between the two
// buffers) are captured once into a CUDA graph and replayed; the autotuner
// times the variants on the live data and the graph is re-captured for the
// one it keeps.  The gradient is one-sided at every domain face, as at the
// domain box of a single run (the box's own_domain bit).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mbg_lowp_types.cuh"

// latched message of a failed creation (mbg_capi.cu), read by mbg_last_error(NULL)
void mbg_set_global_error(const std::string& msg);

using namespace mbg;

#define LOWP16(bf, fn, ...) ((bf) ? Lowp16<true>::fn(__VA_ARGS__) : Lowp16<false>::fn(__VA_ARGS__))

struct mbg_batch {
    mbg_params p{};
    cudaStream_t s = nullptr;
    bool own_stream = false;
    bool bf = false;
    std::string err;
    int ndom = 0;
    std::vector<DevBox> hbox;          // padded layout; hoff = host offset
    long long N = 0, NV = 0;
    std::vector<void*> allocs;
    DevBox* d_box = nullptr;
    uint8_t* d_flags = nullptr;
    Phys32* d_phys = nullptr;
    u16 *f[2] = {nullptr, nullptr}, *g[2] = {nullptr, nullptr};
    float* qs = nullptr;
    double* tmp = nullptr;
    HaloCell* halo = nullptr;
    long long nhalo = 0;
    Tile* tiles = nullptr;             // 128-cell tiles (two-pass variant 3, state transfer)
    int ntiles = 0;
    Tile* ptiles = nullptr;            // variant 0: pair tiles and per-cell tiles (step_tiles)
    int nptiles = 0;
    Tile* ctiles = nullptr;
    int nctiles = 0;
    FusedTile* ftiles[2] = {nullptr, nullptr};
    int nftiles[2] = {0, 0};
    int fgrid = 0;                     // persistent grid of the fused variants
    LowpK hk[2];
    LowpK* dk = nullptr;
    CodecTab ct;
    Lattice<float> lat;
    int cur = 0;
    int variant = 0;
    double variant_ms[4] = {0, 0, 0, 0};
    cudaGraphExec_t graph = nullptr;
    long long launches = 0;
    long long graph_launches = 0;      // kernel launches of one replay of the two-step graph
};

static mbg_status bfail(mbg_batch* b, mbg_status st, const std::string& m)
{
    if (b) b->err = m;
    return st;
}

#define BCUDA(call)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return bfail(b, MBG_ECUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
static mbg_status balloc(mbg_batch* b, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return MBG_OK;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess)
        return bfail(b, e == cudaErrorMemoryAllocation ? MBG_ENOMEM : MBG_ECUDA,
                     std::string("cudaMalloc (batch): ") + cudaGetErrorString(e));
    b->allocs.push_back(*p);
    return MBG_OK;
}

static void drop_graph(mbg_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

// one step from buffer cur into the other (launches only; the caller flips)
static void launch_step(mbg_batch* b, int cur)
{
    const LowpK* k = b->dk + cur;
    LOWP16(b->bf, halo_periodic, k, b->halo, b->nhalo, b->s);
    if (b->variant == 0 || b->variant == 3) {
        // no pad of Q_corr: every domain face is one-sided
        const QPtrs qp = make_qptrs(b->f[cur], b->g[cur], b->f[1 - cur], b->g[1 - cur], b->N);
        const bool pairs = b->variant == 0;
        PairLists pl;
        if (pairs) {
            pl.pair = b->ptiles;
            pl.npair = b->nptiles;
        }
        b->launches += 1 + LOWP16(b->bf, two_pass, k, b->ct, b->lat, pairs ? b->ctiles : b->tiles,
                                  pairs ? b->nctiles : b->ntiles, pl, QPad{},
                                  b->qs, qp, !pairs, b->s);
    } else {
        const int v = b->variant - 1;
        LOWP16(b->bf, fused, k, b->ct, b->lat, b->ftiles[v], b->nftiles[v], std::min(b->fgrid, b->nftiles[v]), b->s);
        b->launches += 2;
    }
}

extern "C" {

mbg_status mbg_batch_create(const mbg_params* common, int ndom, const mbg_domain* doms, void* stream,
                            mbg_batch** out)
{
    if (!common || !doms || !out || ndom <= 0) {
        mbg_set_global_error("mbg_batch_create: null argument or no domains");
        return MBG_EINVAL;
    }
    *out = nullptr;
    if (common->precision != MBG_FP32C_F16S && common->precision != MBG_FP32C_BF16S) {
        mbg_set_global_error("mbg_batch_create: batched domains use a 16-bit form (FP64: one context per domain)");
        return MBG_EINVAL;
    }
    for (int i = 0; i < ndom; ++i)
        for (int d = 0; d < 3; ++d)
            if (doms[i].n_cell[d] < 2 || !(doms[i].prob_hi[d] > doms[i].prob_lo[d]) || doms[i].n_cell[d] > 4096) {
                mbg_set_global_error("mbg_batch_create: domain " + std::to_string(i) + " has an invalid extent");
                return MBG_EINVAL;
            }
    mbg_batch* b = new mbg_batch();
    b->p = *common;
    b->ndom = ndom;
    b->bf = common->precision == MBG_FP32C_BF16S;
    if (stream) {
        b->s = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess) {
            delete b;
            mbg_set_global_error("mbg_batch_create: cudaStreamCreate failed");
            return MBG_ECUDA;
        }
        b->own_stream = true;
    }
    // boxes: one per domain, host order = domain order
    b->hbox.resize(ndom);
    std::vector<Phys32> phys(ndom);
    long long hoff = 0, foff = 0;
    for (int i = 0; i < ndom; ++i) {
        DevBox& B = b->hbox[i];
        for (int d = 0; d < 3; ++d) {
            B.lo[d] = 0;
            B.n[d] = doms[i].n_cell[d];
        }
        B.hoff = hoff;
        B.foff = foff;
        B.goff = -1;
        B.all_fluid = 1;
        B.vfluid = 1;
        B.phys = i;
        B.own_domain = 1;
        hoff += (long long)B.n[0] * B.n[1] * B.n[2];
        foff += (long long)(B.n[0] + 6) * (B.n[1] + 6) * (B.n[2] + 6);
        mbg_params pi = *common;
        pi.nu = doms[i].nu;
        pi.alpha = doms[i].alpha;
        double idx[3];
        for (int d = 0; d < 3; ++d) idx[d] = 1.0 / ((doms[i].prob_hi[d] - doms[i].prob_lo[d]) / doms[i].n_cell[d]);
        phys[i] = phys32(pi, common->dt_outer, idx);
    }
    b->NV = hoff;
    b->N = pad_boxes(b->hbox);
    if (b->N >= (1LL << 31)) {
        mbg_set_global_error("mbg_batch_create: more than 2^31 padded cells");
        mbg_batch_destroy(b);
        return MBG_EINVAL;
    }
    const std::vector<HaloCell> halo = halo_cells(b->hbox);
    b->nhalo = (long long)halo.size();
    std::vector<Tile> tiles;
    for (int i = 0; i < ndom; ++i) {
        const long long vol = (long long)b->hbox[i].n[0] * b->hbox[i].n[1] * b->hbox[i].n[2];
        for (long long s0 = 0; s0 < vol; s0 += TILE_CELLS) tiles.push_back(Tile{i, (int)s0});
    }
    b->ntiles = (int)tiles.size();
    const StepTiles st_tiles = step_tiles(b->hbox, nullptr);   // every domain is fluid: pairs or per-cell
    const std::vector<Tile>& ptiles = st_tiles.pair;
    const std::vector<Tile>& ctiles = st_tiles.cell;
    b->nptiles = (int)ptiles.size();
    b->nctiles = (int)ctiles.size();
    mbg_status st = MBG_OK;
    // domains in decreasing size, so that the persistent grid's strided walk
    // through the work list takes the largest first
    std::vector<int> order(ndom);
    for (int i = 0; i < ndom; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const DevBox &A = b->hbox[a], &C = b->hbox[c];
        return (long long)A.n[0] * A.n[1] * A.n[2] > (long long)C.n[0] * C.n[1] * C.n[2];
    });
    std::vector<DevBox> sorted(ndom);
    for (int i = 0; i < ndom; ++i) sorted[i] = b->hbox[order[i]];
    auto fill = [&]() -> mbg_status {
        mbg_status s2;
        if ((s2 = balloc(b, &b->d_box, ndom)) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->d_flags, (size_t)foff)) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->d_phys, ndom)) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->halo, halo.size())) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->tiles, tiles.size())) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->ptiles, ptiles.size())) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->ctiles, ctiles.size())) != MBG_OK) return s2;
        for (int v = 0; v < 2; ++v) {
            std::vector<FusedTile> ft = fused_tiles(sorted, FUSED_ZC[v]);
            for (FusedTile& t : ft) t.box = order[t.box];
            b->nftiles[v] = (int)ft.size();
            if ((s2 = balloc(b, &b->ftiles[v], ft.size())) != MBG_OK) return s2;
            if (cudaMemcpyAsync(b->ftiles[v], ft.data(), ft.size() * sizeof(FusedTile), cudaMemcpyHostToDevice,
                                b->s) != cudaSuccess)
                return bfail(b, MBG_ECUDA, "batch: upload of the work list failed");
            if (cudaStreamSynchronize(b->s) != cudaSuccess) return bfail(b, MBG_ECUDA, "batch: upload failed");
        }
        for (int i = 0; i < 2; ++i) {
            if ((s2 = balloc(b, &b->f[i], (size_t)b->N * NQ)) != MBG_OK) return s2;
            if ((s2 = balloc(b, &b->g[i], (size_t)b->N * NQ)) != MBG_OK) return s2;
        }
        if ((s2 = balloc(b, &b->qs, (size_t)b->N * 3)) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->tmp, (size_t)b->NV * NQ)) != MBG_OK) return s2;
        if ((s2 = balloc(b, &b->dk, 2)) != MBG_OK) return s2;
        return MBG_OK;
    };
    if ((st = fill()) != MBG_OK) {
        mbg_set_global_error(b->err);
        mbg_batch_destroy(b);
        return st;
    }
    std::vector<uint8_t> flags((size_t)foff, FL_FLUID);
    cudaStream_t s = b->s;
    bool ok = cudaMemcpyAsync(b->d_box, b->hbox.data(), ndom * sizeof(DevBox), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b->d_flags, flags.data(), flags.size(), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(b->d_phys, phys.data(), ndom * sizeof(Phys32), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b->halo, halo.data(), halo.size() * sizeof(HaloCell), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b->tiles, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              (ptiles.empty() || cudaMemcpyAsync(b->ptiles, ptiles.data(), ptiles.size() * sizeof(Tile),
                                                 cudaMemcpyHostToDevice, s) == cudaSuccess) &&
              (ctiles.empty() || cudaMemcpyAsync(b->ctiles, ctiles.data(), ctiles.size() * sizeof(Tile),
                                                 cudaMemcpyHostToDevice, s) == cudaSuccess);
    for (int i = 0; i < 2 && ok; ++i)
        ok = cudaMemsetAsync(b->f[i], 0xFF, (size_t)b->N * NQ * 2, s) == cudaSuccess &&
             cudaMemsetAsync(b->g[i], 0xFF, (size_t)b->N * NQ * 2, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(b->qs, 0, (size_t)b->N * 3 * sizeof(float), s) == cudaSuccess;
    // constant blocks of the two parities
    b->ct = make_codec(*common);
    b->lat = make_lattice<float>();
    const double idx0[3] = {1.0, 1.0, 1.0};
    for (int a = 0; a < 2 && ok; ++a) {
        LowpK& k = b->hk[a];
        std::memset(&k, 0, sizeof(k));
        k.L.box = b->d_box;
        k.L.nbox = ndom;
        for (int d = 0; d < 3; ++d) {
            k.L.dlo[d] = -(1 << 29);
            k.L.dhi[d] = 1 << 29;
            k.L.per[d] = 0;
            k.L.G[d] = 1;
            k.L.nb[d] = 0;
        }
        k.L.omap = nullptr;
        k.L.N = b->N;
        k.L.NG = 0;
        k.L.flags = b->d_flags;
        k.ph = phys32(*common, common->dt_outer, idx0);
        k.ct = b->ct;
        k.lat64 = make_lattice<double>();
        k.s.f = b->f[a];
        k.s.g = b->g[a];
        k.fA = b->f[a];
        k.gA = b->g[a];
        k.fB = b->f[1 - a];
        k.gB = b->g[1 - a];
        k.phys = b->d_phys;
    }
    ok = ok && cudaMemcpyAsync(b->dk, b->hk, 2 * sizeof(LowpK), cudaMemcpyHostToDevice, s) == cudaSuccess &&
         cudaStreamSynchronize(s) == cudaSuccess;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    b->fgrid = std::max(1, nsm) * LOWP16(b->bf, fused_blocks_per_sm);
    if (!ok) {
        mbg_set_global_error("mbg_batch_create: device setup failed");
        mbg_batch_destroy(b);
        return MBG_ECUDA;
    }
    *out = b;
    return MBG_OK;
}

mbg_status mbg_batch_cells(const mbg_batch* b, long long* ncells)
{
    if (!b || !ncells) return MBG_EINVAL;
    *ncells = b->NV;
    return MBG_OK;
}

mbg_status mbg_batch_set_state(mbg_batch* b, const double* f, const double* g)
{
    if (!b || !f || !g) return MBG_EINVAL;
    for (int lat = 0; lat < 2; ++lat) {
        const double* src = lat ? g : f;
        long long off = 0;
        for (int i = 0; i < b->ndom; ++i) {
            const DevBox& B = b->hbox[i];
            const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
            BCUDA(cudaMemcpy2DAsync(b->tmp + B.hoff, b->NV * sizeof(double), src + off * NQ, vol * sizeof(double),
                                    vol * sizeof(double), NQ, cudaMemcpyHostToDevice, b->s));
            off += vol;
        }
        LOWP16(b->bf, encode, b->dk + b->cur, b->tiles, b->ntiles, b->tmp, b->NV, lat ? b->g[b->cur] : b->f[b->cur],
               lat, b->s);
        ++b->launches;
    }
    BCUDA(cudaStreamSynchronize(b->s));
    return MBG_OK;
}

mbg_status mbg_batch_get_state(mbg_batch* b, double* f, double* g)
{
    if (!b || !f || !g) return MBG_EINVAL;
    for (int lat = 0; lat < 2; ++lat) {
        double* dst = lat ? g : f;
        LOWP16(b->bf, decode, b->dk + b->cur, b->tiles, b->ntiles, lat ? b->g[b->cur] : b->f[b->cur], b->NV, b->tmp,
               lat, b->s);
        ++b->launches;
        long long off = 0;
        for (int i = 0; i < b->ndom; ++i) {
            const DevBox& B = b->hbox[i];
            const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
            BCUDA(cudaMemcpy2DAsync(dst + off * NQ, vol * sizeof(double), b->tmp + B.hoff, b->NV * sizeof(double),
                                    vol * sizeof(double), NQ, cudaMemcpyDeviceToHost, b->s));
            off += vol;
        }
        BCUDA(cudaStreamSynchronize(b->s));
    }
    return MBG_OK;
}

mbg_status mbg_batch_get_macro(mbg_batch* b, double* out19)
{
    if (!b || !out19) return MBG_EINVAL;
    double* d = nullptr;
    BCUDA(cudaMallocAsync((void**)&d, (size_t)b->NV * 19 * sizeof(double), b->s));
    LOWP16(b->bf, macro, b->dk + b->cur, b->ct, b->tiles, b->ntiles, d, b->s);
    ++b->launches;
    cudaError_t e = cudaMemcpyAsync(out19, d, (size_t)b->NV * 19 * sizeof(double), cudaMemcpyDeviceToHost, b->s);
    cudaFreeAsync(d, b->s);
    if (e != cudaSuccess) return bfail(b, MBG_ECUDA, std::string("mbg_batch_get_macro: ") + cudaGetErrorString(e));
    BCUDA(cudaStreamSynchronize(b->s));
    return MBG_OK;
}

mbg_status mbg_batch_step(mbg_batch* b, int nsteps)
{
    if (!b || nsteps < 0) return MBG_EINVAL;
    int left = nsteps;
    if (left >= 2 && !b->graph && b->cur == 0) {
        // capture two steps (0 -> 1 -> 0) once
        cudaGraph_t gr = nullptr;
        BCUDA(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
        const long long l0 = b->launches;
        launch_step(b, 0);
        launch_step(b, 1);
        b->graph_launches = b->launches - l0;
        b->launches = l0;
        cudaError_t e = cudaStreamEndCapture(b->s, &gr);
        if (e != cudaSuccess) return bfail(b, MBG_ECUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return bfail(b, MBG_ECUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
        }
    }
    while (left > 0) {
        if (left >= 2 && b->graph && b->cur == 0) {
            BCUDA(cudaGraphLaunch(b->graph, b->s));
            b->launches += b->graph_launches;
            left -= 2;
        } else {
            launch_step(b, b->cur);
            b->cur = 1 - b->cur;
            --left;
        }
    }
    BCUDA(cudaGetLastError());
    return MBG_OK;
}

mbg_status mbg_batch_autotune(mbg_batch* b, int reps)
{
    if (!b || reps < 1) return MBG_EINVAL;
    cudaEvent_t e0, e1;
    BCUDA(cudaEventCreate(&e0));
    BCUDA(cudaEventCreate(&e1));
    const int keep = b->variant;
    double best = 0;
    int best_v = keep;
    for (int v = 0; v < 4; ++v) {
        b->variant = v;
        launch_step(b, b->cur);   // warm-up; the parity is not flipped, so the state is unchanged
        cudaEventRecord(e0, b->s);
        for (int r = 0; r < reps; ++r) launch_step(b, b->cur);
        cudaEventRecord(e1, b->s);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            b->variant = keep;
            return bfail(b, MBG_ECUDA, "mbg_batch_autotune: a trial step failed");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        b->variant_ms[v] = ms / reps;
        if (v == 0 || b->variant_ms[v] < best) {
            best = b->variant_ms[v];
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->variant = best_v;
    drop_graph(b);
    return MBG_OK;
}

mbg_status mbg_batch_tuning(mbg_batch* b, int* variant, double ms[4])
{
    if (!b || !variant || !ms) return MBG_EINVAL;
    *variant = b->variant;
    for (int v = 0; v < 4; ++v) ms[v] = b->variant_ms[v];
    return MBG_OK;
}

mbg_status mbg_batch_synchronize(mbg_batch* b)
{
    if (!b) return MBG_EINVAL;
    BCUDA(cudaStreamSynchronize(b->s));
    return MBG_OK;
}

long long mbg_batch_launch_count(const mbg_batch* b) { return b ? b->launches : 0; }

void* mbg_batch_stream(const mbg_batch* b) { return b ? (void*)b->s : nullptr; }

const char* mbg_batch_last_error(const mbg_batch* b) { return b ? b->err.c_str() : ""; }

void mbg_batch_destroy(mbg_batch* b)
{
    if (!b) return;
    if (b->s) cudaStreamSynchronize(b->s);
    drop_graph(b);
    for (void* p : b->allocs) cudaFree(p);
    if (b->own_stream && b->s) cudaStreamDestroy(b->s);
    delete b;
}

}  // extern "C"
