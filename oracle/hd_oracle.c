/*
 * hd_oracle.c -- CPU oracle for the dilation-based Hausdorff distance.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against.  Only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark load it; the library itself never links or calls it.
 *
 * Parity pins (what makes this oracle trustworthy):
 *   - or_forbench() restates the reference's own algorithm, the host loop of
 *     forBench/HausdorffDistance.cu:146-172 around the `dilate` kernel of
 *     forBench/HausdorffDistance.cu:21-98, on host byte arrays.
 *   - or_bfs_dt() is an independent exact method (multi-source breadth-first
 *     search over the same structuring element inside the same volume).
 *   - or_bruteforce_l1() is the definition itself for the 6-neighbour element
 *     (nearest-voxel Manhattan distance), used on small volumes.
 *   - The reference's `dilate` kernel compiled from its own source and run on
 *     a GPU (oracle/ref_kernel.cpp) gives golden vectors for the shipped
 *     18-neighbour element; tests/golden holds fixtures checked by all of the
 *     above.
 *
 * Structuring elements (forBench/HausdorffDistance.cuh:7-8 select them):
 *   OR_SE6   IS_3D 1, CHEBYSHEV 0: the 6 face neighbours
 *            (forBench/HausdorffDistance.cu:35-42).
 *   OR_SE18  IS_3D 1, CHEBYSHEV 1 (the shipped default): the 6 face neighbours,
 *            the 4 in-plane xy diagonals (:46-49) and the 8 3D corners (:51-58).
 *            The 8 xz / yz edge neighbours are NOT part of it.
 *
 * Per-voxel distance (the average-HD ingredient) follows hello.cu:1588-1625:
 * a voxel of the other mask gets the iteration at which the dilated mask first
 * covers it; overlap voxels get 0.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { OR_SE6 = 0, OR_SE18 = 1 };
enum { OR_OK = 0, OR_EMPTY = 1, OR_BAD = 2, OR_OOM = 3, OR_ITER = 7 };

typedef struct {
    int32_t hd;         /* max(hd_ab, hd_ba) */
    int32_t iterations; /* loop trips of the restated host loop */
    uint64_t sum_ab;    /* sum over a in A of d(a, B) */
    uint64_t sum_ba;    /* sum over b in B of d(b, A) */
    uint64_t n_a, n_b, n_a_not_b, n_b_not_a;
    double avg_hd;      /* (sum_ab + sum_ba) / (n_a + n_b) */
    int32_t status;
    int32_t hd_ab;      /* max over a in A of d(a, B) */
    int32_t hd_ba;      /* max over b in B of d(b, A) */
    int32_t pad;
} or_result;

/* Offsets of the structuring elements, in (dx, dy, dz).  The order mirrors
 * the order of the writes in forBench/HausdorffDistance.cu:35-58. */
static const int8_t SE_OFFS[18][3] = {
    { 1, 0, 0}, {-1, 0, 0}, { 0, 1, 0}, { 0,-1, 0}, { 0, 0, 1}, { 0, 0,-1},
    { 1,-1, 0}, {-1,-1, 0}, { 1, 1, 0}, {-1, 1, 0},
    { 1,-1, 1}, {-1,-1, 1}, { 1, 1, 1}, {-1, 1, 1},
    { 1,-1,-1}, {-1,-1,-1}, { 1, 1,-1}, {-1, 1,-1},
};

static int se_count(int se) { return se == OR_SE18 ? 18 : 6; }

static void count_masks(const uint8_t* A, const uint8_t* B, size_t N, or_result* r) {
    uint64_t na = 0, nb = 0, nab = 0;
    for (size_t i = 0; i < N; ++i) {
        int a = A[i] != 0, b = B[i] != 0;
        na += a; nb += b; nab += (a & b);
    }
    r->n_a = na; r->n_b = nb; r->n_a_not_b = na - nab; r->n_b_not_a = nb - nab;
}

static void finish_avg(or_result* r) {
    uint64_t den = r->n_a + r->n_b;
    r->avg_hd = den ? (double)(r->sum_ab + r->sum_ba) / (double)den : 0.0;
    r->hd = r->hd_ab > r->hd_ba ? r->hd_ab : r->hd_ba;
}

/* ---------------------------------------------------------------------------
 * or_forbench: restatement of HausdorffDistance::computeDistance
 * (forBench/HausdorffDistance.cu:101-187) with the `dilate` kernel
 * (forBench/HausdorffDistance.cu:21-98) executed on the CPU.
 *
 * nthreads == 1: the serial form, written as the reference writes it: every
 *   set voxel of the Read buffer scatters `true` into its in-volume
 *   neighbours of the Write buffer (:24-91), the cover test of :96 is ANDed
 *   over all voxels, then Write is copied to Read (:161-162) and the loop
 *   counter is incremented (:171).
 * nthreads > 1: the same scatter and copy with the z-planes split across
 *   OpenMP threads (stores into another thread's planes are relaxed atomic
 *   byte stores of the same value 1).
 *
 * The reference loops forever when exactly one mask is empty (the test at :96
 * can never become true); here that case returns OR_EMPTY at once.  Each loop
 * trip also records, for every voxel of the other mask that the current
 * dilation covers for the first time, the trip index as its distance
 * (hello.cu:1616-1618 records the same iteration number).
 * hist_ab[k] / hist_ba[k] (length hist_len, may be NULL) count the voxels of
 * A (resp. B) whose distance is k.
 * ------------------------------------------------------------------------- */
int or_forbench(const uint8_t* A, const uint8_t* B, int W, int H, int D, int se,
                int nthreads, or_result* out, uint64_t* hist_ab, uint64_t* hist_ba,
                int hist_len) {
    if (!A || !B || !out || W <= 0 || H <= 0 || D <= 0) return OR_BAD;
    if (se != OR_SE6 && se != OR_SE18) return OR_BAD;
    memset(out, 0, sizeof(*out));
    const size_t N = (size_t)W * H * D;
    const size_t WH = (size_t)W * H;
    count_masks(A, B, N, out);
    if (hist_ab) memset(hist_ab, 0, sizeof(uint64_t) * (size_t)hist_len);
    if (hist_ba) memset(hist_ba, 0, sizeof(uint64_t) * (size_t)hist_len);
    if (out->n_a == 0 && out->n_b == 0) { out->status = OR_OK; finish_avg(out); return OR_OK; }
    if (out->n_a == 0 || out->n_b == 0) {
        out->status = OR_EMPTY; out->hd = -1; out->hd_ab = out->hd_ba = -1;
        out->avg_hd = __builtin_nan("");
        return OR_EMPTY;
    }
    uint8_t* buf = (uint8_t*)malloc(6 * N);
    if (!buf) return OR_OOM;
    uint8_t *r1 = buf, *w1 = buf + N, *r2 = buf + 2 * N, *w2 = buf + 3 * N;
    uint8_t *cov_a = buf + 4 * N, *cov_b = buf + 5 * N; /* first-cover markers */
    for (size_t i = 0; i < N; ++i) {
        r1[i] = w1[i] = A[i] != 0;
        r2[i] = w2[i] = B[i] != 0;
    }
    memset(cov_a, 0, 2 * N);
    const int nse = se_count(se);
    const int max_trips = W + H + D + 2; /* the SE6 / SE18 diameter bounds HD */
    int distance = -1, finished = 0, status = OR_OK;
    uint64_t sum_ab = 0, sum_ba = 0;
    int hd_ab = 0, hd_ba = 0;
    if (nthreads <= 1) {
        while (!finished) {
            const int j = distance + 1; /* Read buffers hold the j-th dilation */
            finished = 1;
            /* cover test (:96) and first-cover bookkeeping */
            uint64_t new_a = 0, new_b = 0;
            for (size_t id = 0; id < N; ++id) {
                const int i1 = A[id] != 0, i2 = B[id] != 0;
                if (i2 && r1[id] && !cov_b[id]) { cov_b[id] = 1; ++new_b; }
                if (i1 && r2[id] && !cov_a[id]) { cov_a[id] = 1; ++new_a; }
                finished &= (r2[id] || !i1) && (r1[id] || !i2);
            }
            sum_ab += (uint64_t)j * new_a; sum_ba += (uint64_t)j * new_b;
            if (new_a) hd_ab = j;
            if (new_b) hd_ba = j;
            if (hist_ab && j < hist_len) hist_ab[j] += new_a;
            if (hist_ba && j < hist_len) hist_ba[j] += new_b;
            /* dilate (:21-91): scatter into the Write buffers */
            for (int z = 0; z < D; ++z)
                for (int y = 0; y < H; ++y)
                    for (int x = 0; x < W; ++x) {
                        const size_t id = (size_t)z * WH + (size_t)y * W + x;
                        const int s1 = r1[id], s2 = r2[id];
                        if (!s1 && !s2) continue;
                        for (int s = 0; s < nse; ++s) {
                            const int nx = x + SE_OFFS[s][0], ny = y + SE_OFFS[s][1],
                                      nz = z + SE_OFFS[s][2];
                            if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
                            const size_t nid = (size_t)nz * WH + (size_t)ny * W + nx;
                            if (s1) w1[nid] = 1;
                            if (s2) w2[nid] = 1;
                        }
                    }
            /* Write -> Read (:161-162), then distance++ (:171) */
            memcpy(r1, w1, N);
            memcpy(r2, w2, N);
            ++distance;
            if (distance > max_trips) { status = OR_ITER; break; }
        }
    } else {
#ifdef _OPENMP
        omp_set_num_threads(nthreads);
#endif
        while (!finished) {
            const int j = distance + 1;
            uint64_t new_a = 0, new_b = 0;
            int fin = 1;
#pragma omp parallel for reduction(+ : new_a, new_b) reduction(&& : fin) schedule(static)
            for (int z = 0; z < D; ++z) {
                for (size_t id = (size_t)z * WH; id < (size_t)(z + 1) * WH; ++id) {
                    const int i1 = A[id] != 0, i2 = B[id] != 0;
                    if (i2 && r1[id] && !cov_b[id]) { cov_b[id] = 1; ++new_b; }
                    if (i1 && r2[id] && !cov_a[id]) { cov_a[id] = 1; ++new_a; }
                    fin = fin && (r2[id] || !i1) && (r1[id] || !i2);
                }
            }
            finished = fin;
            sum_ab += (uint64_t)j * new_a; sum_ba += (uint64_t)j * new_b;
            if (new_a) hd_ab = j;
            if (new_b) hd_ba = j;
            if (hist_ab && j < hist_len) hist_ab[j] += new_a;
            if (hist_ba && j < hist_len) hist_ba[j] += new_b;
            /* dilate: the scatter of :24-91 split over z-planes; writes that
             * cross into a neighbouring thread's planes are relaxed atomic
             * byte stores of 1 (all writers store the same value). */
#pragma omp parallel for schedule(static)
            for (int z = 0; z < D; ++z)
                for (int y = 0; y < H; ++y)
                    for (int x = 0; x < W; ++x) {
                        const size_t id = (size_t)z * WH + (size_t)y * W + x;
                        const int s1 = r1[id], s2 = r2[id];
                        if (!s1 && !s2) continue;
                        for (int s = 0; s < nse; ++s) {
                            const int nx = x + SE_OFFS[s][0], ny = y + SE_OFFS[s][1],
                                      nz = z + SE_OFFS[s][2];
                            if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
                            const size_t nid = (size_t)nz * WH + (size_t)ny * W + nx;
                            if (s1) __atomic_store_n(&w1[nid], (uint8_t)1, __ATOMIC_RELAXED);
                            if (s2) __atomic_store_n(&w2[nid], (uint8_t)1, __ATOMIC_RELAXED);
                        }
                    }
            /* Write -> Read */
#pragma omp parallel for schedule(static)
            for (int z = 0; z < D; ++z) {
                memcpy(r1 + (size_t)z * WH, w1 + (size_t)z * WH, WH);
                memcpy(r2 + (size_t)z * WH, w2 + (size_t)z * WH, WH);
            }
            ++distance;
            if (distance > max_trips) { status = OR_ITER; break; }
        }
    }
    free(buf);
    out->iterations = distance + 1;
    out->sum_ab = sum_ab; out->sum_ba = sum_ba;
    out->hd_ab = hd_ab; out->hd_ba = hd_ba;
    out->status = status;
    finish_avg(out);
    /* the reference returns the loop counter: it must equal max(hd_ab, hd_ba) */
    if (status == OR_OK && out->hd != distance) out->status = OR_BAD;
    return out->status;
}

/* ---------------------------------------------------------------------------
 * or_bfs_dt: exact geodesic distance transform of `src` under the element
 * `se` inside the W x H x D volume, by multi-source breadth-first search.
 * dist[v] = number of dilations of src needed to cover v, -1 if never covered
 * (only possible when src is empty).  Independent of the restatement above.
 * ------------------------------------------------------------------------- */
int or_bfs_dt(const uint8_t* src, int W, int H, int D, int se, int32_t* dist) {
    if (!src || !dist || W <= 0 || H <= 0 || D <= 0) return OR_BAD;
    if (se != OR_SE6 && se != OR_SE18) return OR_BAD;
    const size_t N = (size_t)W * H * D, WH = (size_t)W * H;
    int64_t* q = (int64_t*)malloc(sizeof(int64_t) * (N ? N : 1));
    if (!q) return OR_OOM;
    size_t head = 0, tail = 0;
    for (size_t i = 0; i < N; ++i) {
        if (src[i]) { dist[i] = 0; q[tail++] = (int64_t)i; }
        else dist[i] = -1;
    }
    const int nse = se_count(se);
    while (head < tail) {
        const int64_t id = q[head++];
        const int z = (int)(id / (int64_t)WH);
        const int rem = (int)(id - (int64_t)z * (int64_t)WH);
        const int y = rem / W, x = rem - y * W;
        const int32_t nd = dist[id] + 1;
        for (int s = 0; s < nse; ++s) {
            const int nx = x + SE_OFFS[s][0], ny = y + SE_OFFS[s][1], nz = z + SE_OFFS[s][2];
            if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
            const size_t nid = (size_t)nz * WH + (size_t)ny * W + nx;
            if (dist[nid] < 0) { dist[nid] = nd; q[tail++] = (int64_t)nid; }
        }
    }
    free(q);
    return OR_OK;
}

/* One direction from a distance transform: over the voxels of `target`,
 * the maximum, the sum and the histogram of dist_src.  Returns OR_EMPTY if a
 * target voxel is unreachable. */
static int dt_direction(const int32_t* dist_src, const uint8_t* target, size_t N, int32_t* hd,
                        uint64_t* sum, uint64_t* hist, int hist_len) {
    int32_t m = 0;
    uint64_t s = 0;
    for (size_t i = 0; i < N; ++i) {
        if (!target[i]) continue;
        const int32_t d = dist_src[i];
        if (d < 0) return OR_EMPTY;
        if (d > m) m = d;
        s += (uint64_t)d;
        if (hist && d < hist_len) hist[d] += 1;
    }
    *hd = m; *sum = s;
    return OR_OK;
}

/* HD, sums and counts of a mask pair from the two distance transforms. */
int or_hd_from_dt(const uint8_t* A, const uint8_t* B, const int32_t* dist_a, const int32_t* dist_b,
                  int W, int H, int D, or_result* out, uint64_t* hist_ab, uint64_t* hist_ba,
                  int hist_len) {
    if (!A || !B || !out || W <= 0 || H <= 0 || D <= 0) return OR_BAD;
    memset(out, 0, sizeof(*out));
    const size_t N = (size_t)W * H * D;
    count_masks(A, B, N, out);
    if (hist_ab) memset(hist_ab, 0, sizeof(uint64_t) * (size_t)hist_len);
    if (hist_ba) memset(hist_ba, 0, sizeof(uint64_t) * (size_t)hist_len);
    if (out->n_a == 0 && out->n_b == 0) { finish_avg(out); return OR_OK; }
    if (out->n_a == 0 || out->n_b == 0) {
        out->status = OR_EMPTY; out->hd = out->hd_ab = out->hd_ba = -1;
        out->avg_hd = __builtin_nan("");
        return OR_EMPTY;
    }
    /* d(a, B) comes from the transform of B and vice versa */
    int st = dt_direction(dist_b, A, N, &out->hd_ab, &out->sum_ab, hist_ab, hist_len);
    if (st == OR_OK) st = dt_direction(dist_a, B, N, &out->hd_ba, &out->sum_ba, hist_ba, hist_len);
    out->status = st;
    finish_avg(out);
    out->iterations = out->hd + 1;
    return st;
}

/* Both transforms plus the pair result in one call. */
int or_bfs_pair(const uint8_t* A, const uint8_t* B, int W, int H, int D, int se, or_result* out,
                uint64_t* hist_ab, uint64_t* hist_ba, int hist_len) {
    if (!A || !B || !out || W <= 0 || H <= 0 || D <= 0) return OR_BAD;
    const size_t N = (size_t)W * H * D;
    int32_t* da = (int32_t*)malloc(sizeof(int32_t) * N);
    int32_t* db = (int32_t*)malloc(sizeof(int32_t) * N);
    if (!da || !db) { free(da); free(db); return OR_OOM; }
    int st = or_bfs_dt(A, W, H, D, se, da);
    if (st == OR_OK) st = or_bfs_dt(B, W, H, D, se, db);
    if (st == OR_OK) st = or_hd_from_dt(A, B, da, db, W, H, D, out, hist_ab, hist_ba, hist_len);
    free(da); free(db);
    return st;
}

/* ---------------------------------------------------------------------------
 * or_bruteforce_l1: the definition for the 6-neighbour element.  For every
 * voxel of one mask, the Manhattan distance to the nearest voxel of the other
 * mask.  O(|A| * |B|): small volumes only.
 * ------------------------------------------------------------------------- */
static int32_t* collect(const uint8_t* M, int W, int H, int D, size_t* n) {
    size_t c = 0, N = (size_t)W * H * D;
    for (size_t i = 0; i < N; ++i) c += M[i] != 0;
    int32_t* xyz = (int32_t*)malloc(sizeof(int32_t) * 3 * (c ? c : 1));
    if (!xyz) return NULL;
    size_t k = 0;
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x)
                if (M[(size_t)z * W * H + (size_t)y * W + x]) {
                    xyz[3 * k] = x; xyz[3 * k + 1] = y; xyz[3 * k + 2] = z; ++k;
                }
    *n = c;
    return xyz;
}

static void brute_dir(const int32_t* t, size_t nt, const int32_t* s, size_t ns, int32_t* hd,
                      uint64_t* sum) {
    int32_t m = 0;
    uint64_t acc = 0;
    for (size_t i = 0; i < nt; ++i) {
        int32_t best = INT32_MAX;
        for (size_t j = 0; j < ns && best > 0; ++j) {
            int32_t d = abs(t[3 * i] - s[3 * j]) + abs(t[3 * i + 1] - s[3 * j + 1]) +
                        abs(t[3 * i + 2] - s[3 * j + 2]);
            if (d < best) best = d;
        }
        if (best > m) m = best;
        acc += (uint64_t)best;
    }
    *hd = m; *sum = acc;
}

int or_bruteforce_l1(const uint8_t* A, const uint8_t* B, int W, int H, int D, or_result* out) {
    if (!A || !B || !out || W <= 0 || H <= 0 || D <= 0) return OR_BAD;
    memset(out, 0, sizeof(*out));
    const size_t N = (size_t)W * H * D;
    count_masks(A, B, N, out);
    if (out->n_a == 0 && out->n_b == 0) { finish_avg(out); return OR_OK; }
    if (out->n_a == 0 || out->n_b == 0) {
        out->status = OR_EMPTY; out->hd = out->hd_ab = out->hd_ba = -1;
        out->avg_hd = __builtin_nan("");
        return OR_EMPTY;
    }
    size_t na = 0, nb = 0;
    int32_t* pa = collect(A, W, H, D, &na);
    int32_t* pb = collect(B, W, H, D, &nb);
    if (!pa || !pb) { free(pa); free(pb); return OR_OOM; }
    brute_dir(pa, na, pb, nb, &out->hd_ab, &out->sum_ab);
    brute_dir(pb, nb, pa, na, &out->hd_ba, &out->sum_ba);
    free(pa); free(pb);
    finish_avg(out);
    out->iterations = out->hd + 1;
    return OR_OK;
}

/* ---------------------------------------------------------------------------
 * or_tile_counts: T_k for k = 1..kmax, the number of origin-aligned
 * 32 x 32 x 32 tiles holding at least one voxel v with dist[v] == k, counting
 * only voxels inside the box [x0,x1] x [y0,y1] x [z0,z1].  These are the tiles
 * that step k of an ideal frontier dilation has to touch; the benchmark's
 * algorithmic byte count is built from them.
 * ------------------------------------------------------------------------- */
int or_tile_counts(const int32_t* dist, int W, int H, int D, int x0, int x1, int y0, int y1, int z0,
                   int z1, int kmax, uint64_t* counts) {
    if (!dist || !counts || kmax < 0) return OR_BAD;
    memset(counts, 0, sizeof(uint64_t) * (size_t)(kmax + 1));
    int64_t* stamp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(kmax + 1));
    if (!stamp) return OR_OOM;
    for (int k = 0; k <= kmax; ++k) stamp[k] = -1;
    const int tw = (W + 31) / 32, th = (H + 31) / 32, td = (D + 31) / 32;
    const size_t WH = (size_t)W * H;
    for (int tz = 0; tz < td; ++tz)
        for (int ty = 0; ty < th; ++ty)
            for (int tx = 0; tx < tw; ++tx) {
                const int64_t tid = ((int64_t)tz * th + ty) * tw + tx;
                for (int z = tz * 32; z < tz * 32 + 32 && z < D; ++z) {
                    if (z < z0 || z > z1) continue;
                    for (int y = ty * 32; y < ty * 32 + 32 && y < H; ++y) {
                        if (y < y0 || y > y1) continue;
                        for (int x = tx * 32; x < tx * 32 + 32 && x < W; ++x) {
                            if (x < x0 || x > x1) continue;
                            const int32_t d = dist[(size_t)z * WH + (size_t)y * W + x];
                            if (d >= 1 && d <= kmax && stamp[d] != tid) { stamp[d] = tid; counts[d]++; }
                        }
                    }
                }
            }
    free(stamp);
    return OR_OK;
}
