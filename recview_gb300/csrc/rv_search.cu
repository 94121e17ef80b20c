// Centre search with a learned proposal (no reference counterpart).  The plain method is the
// axis-scan sweep (source/gazoDoc.cpp:1994-2024) on a grid of 2K+1 trial centres, step h, around a
// grid centre (GetAxis's estimate), scored by RvCentreSweep's criterion; it picks the lowest score
// and refines it with a parabola through its neighbours.  The learned search asks the network
// (rv_cnn.cu) for a centre and its uncertainty, reconstructs the 2w+1 grid trials around it and
// walks towards lower scores until the lowest score is confirmed over +-(w+1) grid steps; when
// the grid centre lies outside the first 2w+1 trials, a second walk starts at the grid centre.
// It runs the full sweep when the uncertainty is above sigma_max or the walks exceed 5 (2w+1)
// trials (the criterion keeps disagreeing with the proposal).  Both paths pick the lowest
// evaluated score with the same parabola, so the chosen centre equals the full sweep's whenever
// the walk ends at the grid's lowest score; the final slice is always the plain reconstruction.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "rv_internal.h"

using namespace rv;

extern "C" int RvCentreSearch(RvCentreNet* net, const short* d_sino, int S, int W, int nframes, const char* bInc,
                              const float* fdeg, int s_net, int s_sweep, const float* fFilter, double grid_centre,
                              int half_range, double step, int window, double sigma_max, RvCentreSearchResult* out,
                              void* stream) {
    if (!d_sino || !bInc || !fdeg || !fFilter || !out || S < 1 || W < 4 || nframes < 1 || s_sweep < 0 ||
        s_sweep >= S || half_range < 1 || step <= 0 || window < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreSearch: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = (cudaStream_t)stream;
    memset(out, 0, sizeof(*out));
    out->proposal = NAN;
    out->sigma = NAN;
    std::vector<int> frames;
    for (int f = 0; f < nframes; f++)
        if (bInc[f] & RV_BINC_SAMPLE) frames.push_back(f);
    const int V = (int)frames.size();
    if (V < 2) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvCentreSearch: fewer than two sample frames");
        return RV_ERR_BAD_ARGUMENT;
    }
    int rc = 0;
    // ---- proposal ------------------------------------------------------------------------------
    bool use_net = net != nullptr;
    if (use_net) {
        int f256[256];
        for (int r = 0; r < 256; r++) {
            int i = (int)floor((double)r * V / 256.0 + 0.5);
            if (i >= V) i = V - 1;
            f256[r] = frames[i];
        }
        void* d_x = nullptr;
        if (!cuda_ok(cudaMalloc(&d_x, sizeof(__nv_bfloat16) * 4 * 256 * 512), RV_ERR_DEVICE_OOM, "net input"))
            return RV_ERR_DEVICE_OOM;
        float mu = 0.0f, s = 0.0f;
        rc = RvCentreNetInput(d_sino, S, W, f256, s_net, d_x, stream);
        if (!rc) rc = RvCentreNetForward(net, d_x, 1, &mu, &s, stream);
        cudaFree(d_x);
        if (rc) return rc;
        out->proposal = (W - 1) / 2.0 + 16.0 * mu;
        out->sigma = 16.0 * exp(0.5 * (double)s);
        if (!(out->sigma <= sigma_max)) use_net = false;
    }
    // ---- the sweep slice's sample rows on the host ---------------------------------------------
    std::vector<short> all((size_t)nframes * W), rows((size_t)V * W);
    std::vector<float> vdeg(V);
    if (!cuda_ok(cudaMemcpy2DAsync(all.data(), (size_t)W * 2, d_sino + (size_t)s_sweep * W, (size_t)S * W * 2,
                                   (size_t)W * 2, nframes, cudaMemcpyDeviceToHost, st), RV_ERR_COPY_D2H, "sweep rows") ||
        !cuda_ok(cudaStreamSynchronize(st), RV_ERR_COPY_D2H, "sweep rows"))
        return RV_ERR_COPY_D2H;
    for (int v = 0; v < V; v++) {
        memcpy(&rows[(size_t)v * W], &all[(size_t)frames[v] * W], sizeof(short) * W);
        vdeg[v] = fdeg[frames[v]];
    }
    // ---- trials: scores on the grid, computed once each -------------------------------------------
    const int K = half_range, NG = 2 * K + 1;
    std::vector<double> score(NG, 0.0);
    std::vector<char> have(NG, 0);
    auto centre_of = [&](int k) { return grid_centre + step * k; };
    auto eval = [&](int k0, int k1) -> int {   // the missing grid points of [k0, k1], one batch
        k0 = k0 < -K ? -K : k0;
        k1 = k1 > K ? K : k1;
        std::vector<double> cs;
        std::vector<int> ks;
        for (int k = k0; k <= k1; k++)
            if (!have[k + K]) { cs.push_back(centre_of(k)); ks.push_back(k); }
        if (cs.empty()) return 0;
        std::vector<double> sc(cs.size());
        double unused = 0.0;
        const int r = RvCentreSweep(rows.data(), V, W, 2, vdeg.data(), 0.0f, fFilter, cs.data(), (int)cs.size(),
                                    sc.data(), &unused);
        if (r) return r;
        for (size_t i = 0; i < ks.size(); i++) {
            score[ks[i] + K] = sc[i];
            have[ks[i] + K] = 1;
        }
        out->trials += (int)cs.size();
        return 0;
    };
    bool full = !use_net;
    if (use_net) {
        // A walk starts with 2*window+1 trials around k and moves towards lower scores in steps of
        // window+1 until its lowest score m is confirmed: every grid point within window+1 of m
        // evaluated and none lower (a shallow bump next to the basin does not stop it).  The first
        // walk starts at the proposal; when the grid centre (GetAxis's estimate) lies outside the
        // proposal's first 2*window+1 trials, a second walk starts there.  Both keep the trial cap.
        const int cap = 5 * (2 * window + 1), conf = window + 1;
        auto walk = [&](int kstart) -> int {
            int lo = kstart - window, hi = kstart + window;
            if (lo < -K) { hi += -K - lo; lo = -K; }
            if (hi > K) { lo -= hi - K; hi = K; }
            if (lo < -K) lo = -K;
            int r = eval(lo, hi);
            if (r) return r;
            for (;;) {
                int m = lo;
                for (int k = lo + 1; k <= hi; k++)
                    if (score[k + K] < score[m + K]) m = k;
                if (m == lo && lo > -K) {
                    const int nlo = lo - (window + 1) < -K ? -K : lo - (window + 1);
                    if ((r = eval(nlo, lo - 1))) return r;
                    lo = nlo;
                } else if (m == hi && hi < K) {
                    const int nhi = hi + window + 1 > K ? K : hi + window + 1;
                    if ((r = eval(hi + 1, nhi))) return r;
                    hi = nhi;
                } else {
                    // m has evaluated neighbours on both sides: confirm it over +-conf
                    const int clo = m - conf < -K ? -K : m - conf, chi = m + conf > K ? K : m + conf;
                    if (clo >= lo && chi <= hi) break;
                    if (clo < lo) {
                        if ((r = eval(clo, lo - 1))) return r;
                        lo = clo;
                    }
                    if (chi > hi) {
                        if ((r = eval(hi + 1, chi))) return r;
                        hi = chi;
                    }
                    int m2 = lo;
                    for (int k = lo + 1; k <= hi; k++)
                        if (score[k + K] < score[m2 + K]) m2 = k;
                    if (m2 == m) break;   // confirmed; otherwise keep walking from the lower point
                }
                if (out->trials > cap) { full = true; break; }   // the criterion keeps disagreeing
            }
            return 0;
        };
        int kp = (int)floor((out->proposal - grid_centre) / step + 0.5);
        kp = kp < -K ? -K : (kp > K ? K : kp);
        if ((rc = walk(kp))) return rc;
        if (!full && abs(kp) > window && (rc = walk(0))) return rc;
    }
    if (full) {
        out->fallback = 1;
        if ((rc = eval(-K, K))) return rc;
    }
    // lowest evaluated score (ties: lowest k), parabola through its evaluated neighbours -- the
    // full sweep's rule (RvCentreSweep) on the same grid values
    int m = -K - 1;
    for (int k = -K; k <= K; k++)
        if (have[k + K] && (m < -K || score[k + K] < score[m + K])) m = k;
    double best = centre_of(m);
    if (m > -K && m < K && have[m - 1 + K] && have[m + 1 + K]) {
        const double s0 = score[m - 1 + K], s1 = score[m + K], s2 = score[m + 1 + K];
        const double den = s0 - 2 * s1 + s2;
        const double h0 = centre_of(m) - centre_of(m - 1), h1 = centre_of(m + 1) - centre_of(m);
        if (den > 0 && fabs(h0 - h1) < 1e-9) best = centre_of(m) + 0.5 * h0 * (s0 - s2) / den;
    }
    out->centre = best;
    out->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}
