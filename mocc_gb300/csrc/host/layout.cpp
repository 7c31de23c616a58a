#include "layout.hpp"

#include <algorithm>
#include <numeric>
#include <unordered_map>

namespace mocgpu {

SweepLayout build_sweep_layout(const FlatProblem &f, bool gs, int tracks_per_unit, int max_local, bool interleave,
                               int window_rows)
{
    SweepLayout L;
    const int W = SweepLayout::kLanes;
    if (window_rows < 0 || window_rows % 16 != 0) MOCGPU_THROW(1, "window rows must be a multiple of 16");
    L.window_rows = window_rows;
    if (tracks_per_unit < W) tracks_per_unit = W;
    tracks_per_unit = (tracks_per_unit / W) * W;
    if (max_local > 65535) max_local = 65535;
    const int sets_oct = f.n_sets / 2;
    std::vector<std::vector<int>> phases;
    if (gs) {
        phases.resize(2);
        for (int s = 0; s < f.n_sets; s++) phases[s < sets_oct ? 0 : 1].push_back(s);
    } else {
        phases.resize(1);
        for (int s = 0; s < f.n_sets; s++) phases[0].push_back(s);
    }
    L.n_phases = (int)phases.size();
    int64_t real = 0, padded = 0;
    std::vector<int> mark(f.n_fsr, -1);
    int stamp = 0;
    for (const auto &ph : phases) {
        L.phase_wu_begin.push_back((int)L.wu.size());
        for (int s : ph) {
            int t0 = f.set_first_track[s], t1 = f.set_first_track[s + 1];
            int t = t0;
            while (t < t1) {
                // grow the unit while it stays within both caps
                std::vector<int> tracks, fsrs;
                stamp++;
                while (t < t1 && (int)tracks.size() < tracks_per_unit) {
                    int added = 0;
                    for (int64_t k = f.trk_seg_begin[t]; k < f.trk_seg_begin[t + 1]; k++)
                        if (mark[f.seg_fsr[k]] != stamp) added++;
                    if (!tracks.empty() && (int)fsrs.size() + added > max_local) break;
                    if ((int)fsrs.size() + added > max_local)
                        MOCGPU_THROW(6, "a single track touches more FSRs than a work unit can hold");
                    for (int64_t k = f.trk_seg_begin[t]; k < f.trk_seg_begin[t + 1]; k++)
                        if (mark[f.seg_fsr[k]] != stamp) {
                            mark[f.seg_fsr[k]] = stamp;
                            fsrs.push_back(f.seg_fsr[k]);
                        }
                    tracks.push_back(t);
                    t++;
                }
                WorkUnitHost u;
                u.set = s;
                u.bundle_begin = (int)L.bundle_row.size();
                u.n_local = (int)fsrs.size();
                // longest first, bundles of W
                std::stable_sort(tracks.begin(), tracks.end(), [&](int a, int b) {
                    return (f.trk_seg_begin[a + 1] - f.trk_seg_begin[a]) > (f.trk_seg_begin[b + 1] - f.trk_seg_begin[b]);
                });
                // bundles: the length-sorted tracks dealt round-robin, so the
                // lanes of a bundle have similar lengths (little padding) but
                // are not spatial neighbours, which cross the same FSR in the
                // same row and contend for its tally
                const size_t nb = (tracks.size() + W - 1) / W;
                std::vector<std::vector<int>> groups(nb);
                for (size_t j = 0; j < tracks.size(); j++)
                    groups[interleave ? j % nb : j / W].push_back(tracks[j]);
                int maxrows = 0;
                for (const std::vector<int> &grp : groups)
                    for (int tr : grp)
                        maxrows = std::max<int>(maxrows, (int)(f.trk_seg_begin[tr + 1] - f.trk_seg_begin[tr]));
                // row windows: one table of FSRs per window, local ids per window
                const int wr = (window_rows > 0 && maxrows > window_rows) ? window_rows : std::max(maxrows, 1);
                const int nwin = (maxrows + wr - 1) / wr > 0 ? (maxrows + wr - 1) / wr : 1;
                u.win_begin = (int)L.win.size();
                u.n_win = nwin;
                L.max_windows = std::max(L.max_windows, nwin);
                std::vector<std::unordered_map<int, int>> loc(nwin);
                for (int w = 0; w < nwin; w++) {
                    std::vector<int> wf;
                    std::unordered_map<int, int> count;
                    for (int tr : tracks) {
                        const int64_t a = f.trk_seg_begin[tr];
                        const int n = (int)(f.trk_seg_begin[tr + 1] - a);
                        for (int r = w * wr; r < std::min(n, (w + 1) * wr); r++) count[f.seg_fsr[a + r]]++;
                    }
                    wf.reserve(count.size());
                    for (const auto &kv : count) {
                        wf.push_back(kv.first);
                        // a window's table may take both directions' adds (when
                        // forward and backward warps stage the same window)
                        L.max_hits = std::max(L.max_hits, 2 * kv.second);
                    }
                    std::sort(wf.begin(), wf.end());
                    loc[w].reserve(wf.size() * 2);
                    for (size_t i = 0; i < wf.size(); i++) loc[w][wf[i]] = (int)i;
                    L.win.push_back(RowWindowHost{(int)L.local_fsr.size(), (int)wf.size()});
                    L.local_fsr.insert(L.local_fsr.end(), wf.begin(), wf.end());
                    L.max_local = std::max(L.max_local, (int)wf.size() + 1); // + the padding slot
                }
                for (const std::vector<int> &grp : groups) {
                    int nrows = 0;
                    for (int tr : grp) nrows = std::max<int>(nrows, (int)(f.trk_seg_begin[tr + 1] - f.trk_seg_begin[tr]));
                    L.bundle_row.push_back(L.n_rows);
                    L.bundle_nrows.push_back(nrows);
                    size_t base = L.len.size();
                    L.len.resize(base + (size_t)nrows * W, 0.0);
                    L.lfsr.resize(base + (size_t)nrows * W, 0);
                    // padding entries keep length 0 and point at their window's
                    // padding slot (local id n_local, after its FSRs)
                    for (int r = 0; r < nrows; r++)
                        for (int lane = 0; lane < W; lane++)
                            L.lfsr[base + (size_t)r * W + lane] = (uint16_t)L.win[u.win_begin + r / wr].n_local;
                    for (int lane = 0; lane < W; lane++) {
                        if (lane >= (int)grp.size()) {
                            L.bundle_track.push_back(-1);
                            continue;
                        }
                        int tr = grp[lane];
                        L.bundle_track.push_back(tr);
                        int64_t a = f.trk_seg_begin[tr];
                        int n = (int)(f.trk_seg_begin[tr + 1] - a);
                        for (int r = 0; r < n; r++) {
                            L.len[base + (size_t)r * W + lane] = f.seg_len[a + r];
                            L.lfsr[base + (size_t)r * W + lane] = (uint16_t)loc[r / wr].at(f.seg_fsr[a + r]);
                        }
                        real += n;
                    }
                    padded += (int64_t)nrows * W;
                    L.n_rows += nrows;
                }
                u.n_bundles = (int)L.bundle_row.size() - u.bundle_begin;
                L.wu.push_back(u);
            }
        }
        // longest units first: a single-solve launch has one CTA per unit,
        // dispatched in index order, so the long units start in the first
        // wave and the short ones fill the tail
        auto rows = [&](const WorkUnitHost &u) {
            int mx = 0, sum = 0;
            for (int b = 0; b < u.n_bundles; b++) {
                mx = std::max(mx, L.bundle_nrows[u.bundle_begin + b]);
                sum += L.bundle_nrows[u.bundle_begin + b];
            }
            return std::make_pair(mx, sum);
        };
        std::stable_sort(L.wu.begin() + L.phase_wu_begin.back(), L.wu.end(),
                         [&](const WorkUnitHost &a, const WorkUnitHost &b) { return rows(a) > rows(b); });
    }
    L.phase_wu_begin.push_back((int)L.wu.size());
    L.padding = real ? (double)padded / (double)real - 1.0 : 0.0;
    return L;
}

} // namespace mocgpu
