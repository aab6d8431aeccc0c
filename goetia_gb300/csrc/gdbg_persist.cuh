// Persistent fused hash + insert kernel for packed read batches.
//
// One cooperative launch inserts a whole batch.  Work unit: a warp task =
// up to 32 consecutive k-mers of one read, one k-mer per lane.  The lane
// hashes are produced together: the warp XOR-reduces the K terms of the first
// k-mer's hash (fw = XOR_i rotl(T[s_i], K-1-i), rc = XOR_i rotl(T[comp s_i], i),
// the closed form of CyclicHash eat, cyclichash.h:105-108), then an inclusive
// shuffle scan applies the per-lane roll
//   fw_l = rotl1(fw_{l-1}) ^ rotl_K(T[out]) ^ T[in]          (update, :85-92)
//   rc_l = rotr1(rc_{l-1} ^ rotl_K(T[comp in]) ^ T[comp out])  (reverse_update, :96-101)
// so lane l holds the hash of k-mer p0+l after log2(32) steps.
//
// The batch's tasks are cut into windows.  For each window the grid runs the
// probe phase (read the cells, note the zero ones, claim them in the
// first-touch map), waits at a grid barrier, runs the commit phase (apply the
// inserts, decide which k-mers are new), and waits again.  A window's table
// sectors stay in L2 between the two phases.  The barrier spins with an
// iteration cap (PersistParams::spin_cap, WAIT_CAP by default): when it runs
// out the kernel records GDBG_ERR_BARRIER_TIMEOUT and every block returns.
// The claims of an aborted run are never trusted again: the kernel leaves the
// epoch at 127, so the next run starts by clearing the claims map.
#pragma once
#include "gdbg_kernels.cuh"

namespace gdbg {

constexpr int PBLOCK = 512;

// Grid-wide barrier for a cooperative launch.  Returns false (for every
// thread of the block) when the wait ran past `cap` polls.
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, uint32_t* err, uint32_t cap) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* vgen = bar + 1;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t spins = 0;
            while (*vgen == gen) {
                if (++spins > cap) {
                    atomicOr(err, GDBG_ERR_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Hashes of the k-mers of one warp task; lane l gets k-mer p0 + l.
template <bool CANON>
__device__ __forceinline__ void task_hash(const uint32_t* __restrict__ packed, uint64_t b0,
                                          const HashParams& hp, bool valid, uint32_t lane,
                                          uint64_t& fw, uint64_t& rc) {
    const uint32_t K = hp.K;
    uint64_t sf = 0, sr = 0;
    for (uint32_t i = lane; i < K; i += 32) {
        const uint32_t c = base_at(packed, b0 + i);
        sf ^= rotl64(sym(c), (K - 1u - i) & 63u);
        if (CANON) sr ^= rotl64(sym(3u - c), i & 63u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sf ^= __shfl_xor_sync(0xFFFFFFFFu, sf, o);
        if (CANON) sr ^= __shfl_xor_sync(0xFFFFFFFFu, sr, o);
    }
    uint64_t vf = sf, vr = sr;
    if (lane > 0) {
        vf = 0;
        vr = 0;
        if (valid) {
            const uint32_t out = base_at(packed, b0 + lane - 1);
            const uint32_t in = base_at(packed, b0 + lane + K - 1);
            vf = symk(hp, out) ^ sym(in);
            if (CANON) vr = rotr1(symk(hp, 3u - in) ^ sym(3u - out));
        }
    }
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint64_t yf = __shfl_up_sync(0xFFFFFFFFu, vf, d);
        const uint64_t yr = CANON ? __shfl_up_sync(0xFFFFFFFFu, vr, d) : 0;
        if (lane >= d) {
            vf ^= rotl64(yf, d);
            if (CANON) vr ^= rotl64(yr, 64u - d);
        }
    }
    fw = vf;
    rc = vr;
}

struct TaskInfo {
    uint64_t read, b0, g;
    bool valid;
};

__device__ __forceinline__ TaskInfo task_info(const BatchView& b, uint64_t t, uint32_t lane) {
    TaskInfo ti;
    ti.read = __ldg(b.task_read + t);
    const uint64_t tr = __ldg(b.tofs + ti.read);
    const uint64_t kr = __ldg(b.kofs + ti.read);
    const uint64_t nk = __ldg(b.kofs + ti.read + 1) - kr;
    const uint64_t p0 = (t - tr) * TASK_KMERS;
    ti.b0 = __ldg(b.offsets + ti.read) + p0;
    ti.valid = p0 + lane < nk;
    ti.g = kr + p0 + lane;
    return ti;
}

template <int STORAGE, bool CANON, int NT>
__device__ __forceinline__ void probe_task(const BatchView& b, const HashParams& hp,
                                           const TableParams& tp, const PersistParams& pp,
                                           uint64_t t, uint64_t gws, uint32_t epoch,
                                           unsigned long long& occ) {
    const uint32_t lane = threadIdx.x & 31;
    const TaskInfo ti = task_info(b, t, lane);
    uint64_t fw, rc;
    task_hash<CANON>(b.packed, ti.b0, hp, ti.valid, lane, fw, rc);
    if (!ti.valid) return;
    const uint64_t h = hash_value<CANON>(fw, rc);
    const uint32_t ord = (uint32_t)(ti.g - gws);
    const int n = NT > 0 ? NT : tp.n;
    constexpr int TG = NT > 0 ? NT : 1;
    uint32_t fresh = 0;
    for (int i0 = 0; i0 < n; i0 += TG) {
        uint64_t bin[TG];
        uint32_t word[TG], shift[TG];
#pragma unroll
        for (int k = 0; k < TG; ++k) {
            const int i = i0 + k;
            if (i < n) {
                bin[k] = fastmod(h, tp.p[i], tp.m[i]);
                Cell c = cell_of<STORAGE>(tp, i, bin[k]);
                shift[k] = c.shift;
                word[k] = __ldcg(c.word);
            }
        }
#pragma unroll
        for (int k = 0; k < TG; ++k) {
            const int i = i0 + k;
            if (i < n) {
                if (STORAGE != GDBG_BIT) pp.words[(uint64_t)ord * n + i] = word[k];
                if (cell_value<STORAGE>(word[k], shift[k]) == 0) {
                    fresh |= 1u << i;
                    const uint64_t id = ((uint64_t)i << 32) | bin[k];
                    if (claim_min(pp.claims, pp.claims_mask, epoch, id, ord, pp.err) && i == 0)
                        ++occ;
                }
            }
        }
    }
    pp.fresh[ord] = fresh;
}

template <int STORAGE, bool CANON, int NT>
__device__ __forceinline__ void commit_task(const BatchView& b, const HashParams& hp,
                                            const TableParams& tp, const PersistParams& pp,
                                            uint64_t t, uint64_t gws, uint32_t epoch,
                                            unsigned long long& uniq) {
    const uint32_t lane = threadIdx.x & 31;
    const TaskInfo ti = task_info(b, t, lane);
    uint64_t fw, rc;
    task_hash<CANON>(b.packed, ti.b0, hp, ti.valid, lane, fw, rc);
    uint32_t isnew = 0;
    if (ti.valid) {
        const uint64_t h = hash_value<CANON>(fw, rc);
        const uint32_t ord = (uint32_t)(ti.g - gws);
        const uint32_t fresh = __ldcg(pp.fresh + ord);
        const int n = NT > 0 ? NT : tp.n;
        constexpr int TG = NT > 0 ? NT : 1;
        for (int i0 = 0; i0 < n; i0 += TG) {
            uint64_t bin[TG];
            uint32_t* wp[TG];
            uint32_t shift[TG], guess[TG], prev[TG];
#pragma unroll
            for (int k = 0; k < TG; ++k) {
                const int i = i0 + k;
                if (i < n) {
                    bin[k] = fastmod(h, tp.p[i], tp.m[i]);
                    Cell c = cell_of<STORAGE>(tp, i, bin[k]);
                    wp[k] = c.word;
                    shift[k] = c.shift;
                }
            }
            if (STORAGE == GDBG_BIT) {
                // a bit that was set at the window start stays set: only the
                // zero bits need the OR
#pragma unroll
                for (int k = 0; k < TG; ++k) {
                    const int i = i0 + k;
                    if (i < n && ((fresh >> i) & 1u)) atomicOr(wp[k], 1u << shift[k]);
                }
            } else {
                // first compare-and-swap of every table issued together; a
                // saturated cell stays saturated and needs none
#pragma unroll
                for (int k = 0; k < TG; ++k) {
                    const int i = i0 + k;
                    if (i < n) {
                        guess[k] = __ldcg(pp.words + (uint64_t)ord * n + i);
                        prev[k] = guess[k];
                        if (cell_value<STORAGE>(guess[k], shift[k]) < cell_max<STORAGE>())
                            prev[k] = atomicCAS(wp[k], guess[k], guess[k] + (1u << shift[k]));
                    }
                }
#pragma unroll
                for (int k = 0; k < TG; ++k) {
                    const int i = i0 + k;
                    if (i < n && prev[k] != guess[k])
                        sat_increment<STORAGE>(wp[k], shift[k], prev[k], pp.err);
                }
            }
#pragma unroll
            for (int k = 0; k < TG; ++k) {
                const int i = i0 + k;
                if (i < n && ((fresh >> i) & 1u)) {
                    const uint64_t id = ((uint64_t)i << 32) | bin[k];
                    if (claim_lookup(pp.claims, pp.claims_mask, epoch, id) == ord) isnew = 1;
                }
            }
        }
    }
    const uint32_t cnt = __reduce_add_sync(0xFFFFFFFFu, isnew);
    if (lane == 0 && cnt && pp.n_new) atomicAdd(pp.n_new + ti.read, (unsigned long long)cnt);
    uniq += isnew;
}

template <int STORAGE, bool CANON, int NT>
__global__ void __launch_bounds__(PBLOCK, 2)
k_insert_persistent(BatchView b, HashParams hp, TableParams tp, PersistParams pp) {
    const uint64_t warp = ((uint64_t)blockIdx.x * PBLOCK + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * PBLOCK) >> 5;
    const uint64_t tid = (uint64_t)blockIdx.x * PBLOCK + threadIdx.x;
    const uint64_t n_threads = (uint64_t)gridDim.x * PBLOCK;
    uint64_t n_tasks = __ldg(b.tofs + b.n_reads);
    if (n_tasks > b.task_cap) n_tasks = b.task_cap;
    const uint64_t WT = pp.window_tasks;
    uint32_t epoch = *(volatile uint32_t*)pp.epoch_state;
    const uint32_t cap = pp.spin_cap ? pp.spin_cap : WAIT_CAP;
    unsigned long long uniq = 0, occ = 0;
    bool ok = true;
    for (uint64_t t0 = 0; t0 < n_tasks && ok; t0 += WT) {
        const uint64_t t1 = min(n_tasks, t0 + WT);
        if (++epoch > 127) {
            for (uint64_t i = tid; i <= pp.claims_mask; i += n_threads) pp.claims[i] = 0;
            if (!grid_barrier(pp.bar, pp.err, cap)) { ok = false; break; }
            epoch = 1;
        }
        const uint64_t r0 = __ldg(b.task_read + t0);
        const uint64_t gws = __ldg(b.kofs + r0) + (t0 - __ldg(b.tofs + r0)) * TASK_KMERS;
        for (uint64_t t = t0 + warp; t < t1; t += n_warps)
            probe_task<STORAGE, CANON, NT>(b, hp, tp, pp, t, gws, epoch, occ);
        if (!grid_barrier(pp.bar, pp.err, cap)) { ok = false; break; }
        for (uint64_t t = t0 + warp; t < t1; t += n_warps)
            commit_task<STORAGE, CANON, NT>(b, hp, tp, pp, t, gws, epoch, uniq);
        if (!grid_barrier(pp.bar, pp.err, cap)) { ok = false; break; }
    }
    uniq = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)uniq);
    occ = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)occ);
    if ((threadIdx.x & 31) == 0) {
        if (uniq) atomicAdd(pp.counters + 0, uniq);
        if (occ) atomicAdd(pp.counters + 1, occ);
    }
    if (threadIdx.x == 0) {
        // an aborted run leaves claims of epochs the next run would reuse:
        // epoch 127 makes the next run clear the map before its first window
        if (!ok) atomicExch(pp.epoch_state, 127u);
        else if (blockIdx.x == 0) atomicExch(pp.epoch_state, epoch);
    }
}

}  // namespace gdbg
