// Checkpoint schedules for the adjoint pass (host code, no CUDA).
//
// The reference keeps every snap_dt-th forward snapshot in host memory
// (accu_* arrays filled by gard_fwd_storage2, src/cpu/n_kernel_lib_PSV.cpp,
// read back by fwi_grad2 in the time-reversed call of kernel_PSV,
// src/cpu/n_simulate_PSV.cpp:344-356).  The engine can instead keep forward
// *states* (v, sigma, CPML memories) at the start of some K-step segments and
// recompute the forward from them.  The time axis is split into n segments;
// reversing segment j ("leaf") means: working state = forward state at the
// start of j, recompute j with its snapshots into a segment buffer, then run
// j's adjoint steps.  Reaching the start of j from an earlier checkpoint costs
// forward "advances" of whole segments.
//
// With S state slots (the one at segment 0 included) the fewest advances
// F(n, S) obey
//     F(1, S) = 0,  F(n, 1) = n (n - 1) / 2,
//     F(n, S) = min_{0 < m < n} [ m + F(n - m, S - 1) + F(m, S) ]
// (store a checkpoint m segments on, reverse the right part with one slot
// fewer, then the left part).  This is Griewank's binomial checkpointing
// (A. Griewank, "Achieving logarithmic growth of temporal and spatial
// complexity in reverse automatic differentiation", Optimization Methods
// and Software 1, 1992; A. Griewank and A. Walther, ACM TOMS 26, 2000):
// with beta(s, t) = C(s + t, t) and t the least integer with
// beta(S, t) >= n, F(n, S) = t n - beta(S + 1, t - 1), and every split
//     m = min(beta(S, t - 1), n - beta(S - 1, t - 1))
// is optimal (the left part then needs t - 1 repetitions, the right part t,
// and Pascal's rule gives the total).  With S >= n the schedule saves a
// state at every segment start and never advances: the two-level scheme.
//
// The forward pass that records the traces runs every step anyway; it saves
// the states of the schedule's right spine (segment 0, the first split, the
// split of the remainder ...) on its way, so those advances cost nothing.
#pragma once

#include <vector>

namespace psv {

enum CkOp {
    CK_SAVE_MAIN = 1,  // forward pass: state at the start of `seg` -> slot
    CK_RESTORE = 2,    // slot -> working state
    CK_ADVANCE = 3,    // working state: run segment `seg` forward, no snapshots
    CK_SAVE_WORK = 4,  // working state (at the start of `seg`) -> slot
    CK_REVERSE = 5,    // working state at the start of `seg`: recompute `seg` with
                       // snapshots, then its adjoint steps
};

struct CkAction {
    int op, seg, slot;
};

// A schedule lists every segment advance as an action: schedules with more
// advances than this (a few slots forced on a very long record; 12 bytes an
// action, 0.8 GB here) are refused before they are built.
constexpr long long CK_MAX_ADVANCES = 1LL << 26;

// beta(s, t) = C(s + t, t), saturated at 2^62.
inline long long ck_beta(int s, int t)
{
    if (t < 0 || s < 0) return t < 0 ? 0 : 1;
    long long b = 1;
    const long long cap = 1LL << 62;
    for (int i = 1; i <= t; i++) {
        // b * (s + i) / i is exact: b = C(s + i - 1, i - 1)
        const long long num = s + i;
        if (b > cap / num) return cap;
        b = b * num / i;
    }
    return b;
}

// Least t with beta(s, t) >= n (s >= 1, n >= 1).
inline int ck_reps(long long n, int s)
{
    int t = 0;
    while (ck_beta(s, t) < n) t++;
    return t;
}

// Fewest advances to reverse n segments with s slots (closed form).
inline long long ck_min_advances(long long n, int s)
{
    if (n <= 1) return 0;
    if (s <= 1) return n * (n - 1) / 2;
    const int t = ck_reps(n, s);
    return t * n - ck_beta(s + 1, t - 1);
}

// Segments to advance before the first checkpoint (n >= 2, s >= 2).
inline long long ck_split(long long n, int s)
{
    const int t = ck_reps(n, s);
    long long m = ck_beta(s, t - 1);
    const long long r = n - ck_beta(s - 1, t - 1);
    if (r < m) m = r;
    if (m < 1) m = 1;
    if (m > n - 1) m = n - 1;
    return m;
}

struct CkSchedule {
    std::vector<CkAction> fwd;  // CK_SAVE_MAIN, by increasing segment
    std::vector<CkAction> bwd;  // the adjoint pass
    long long advances = 0;     // CK_ADVANCE actions in bwd
    int slots = 0;              // slots the schedule uses
};

class CkBuilder {
  public:
    CkBuilder(int nseg, int slots) : n_(nseg), S_(slots < 1 ? 1 : slots) {}

    CkSchedule build()
    {
        CkSchedule out;
        if (n_ <= 0) return out;
        pos_.assign(S_, -1);
        for (int k = S_ - 1; k >= 0; k--) free_.push_back(k);
        // right spine: saved by the forward pass
        std::vector<int> spine_slot((size_t)n_, -1);
        {
            int a = 0, S = S_;
            const int c0 = take(0);
            spine_slot[0] = c0;
            out.fwd.push_back({CK_SAVE_MAIN, 0, c0});
            while (n_ - a > 1 && S > 1) {
                const int m = a + (int)ck_split(n_ - a, S);
                const int c = take(m);
                spine_slot[(size_t)m] = c;
                out.fwd.push_back({CK_SAVE_MAIN, m, c});
                a = m;
                S--;
            }
        }
        spine_ = &spine_slot;
        bwd_ = &out.bwd;
        rev(0, n_, spine_slot[0], S_, true);
        for (const CkAction &x : out.bwd) out.advances += x.op == CK_ADVANCE;
        out.slots = used_;
        return out;
    }

  private:
    int n_, S_, used_ = 0, work_ = -1;  // work_: segment the working state starts, or -1
    std::vector<int> pos_, free_;
    const std::vector<int> *spine_ = nullptr;
    std::vector<CkAction> *bwd_ = nullptr;

    int take(int seg)
    {
        const int c = free_.back();
        free_.pop_back();
        pos_[(size_t)c] = seg;
        if (S_ - (int)free_.size() > used_) used_ = S_ - (int)free_.size();
        return c;
    }
    void give(int c)
    {
        pos_[(size_t)c] = -1;
        free_.push_back(c);
    }
    void restore(int c)
    {
        if (work_ == pos_[(size_t)c]) return;  // the working state is already there
        bwd_->push_back({CK_RESTORE, pos_[(size_t)c], c});
        work_ = pos_[(size_t)c];
    }
    void advance(int to)
    {
        for (int j = work_; j < to; j++) bwd_->push_back({CK_ADVANCE, j, -1});
        work_ = to;
    }
    void reverse(int j)
    {
        bwd_->push_back({CK_REVERSE, j, -1});
        work_ = -1;  // left inside segment j
    }

    // Reverse segments [a, e); the state at the start of a is in slot c and
    // S slots (c included) may be in use.
    void rev(int a, int e, int c, int S, bool spine)
    {
        if (e - a == 1) {
            restore(c);
            reverse(a);
            return;
        }
        if (S <= 1) {
            for (int j = e - 1; j >= a; j--) {
                restore(c);
                advance(j);
                reverse(j);
            }
            return;
        }
        const int m = a + (int)ck_split(e - a, S);
        int c2;
        if (spine) {
            c2 = (*spine_)[(size_t)m];
        } else {
            restore(c);
            advance(m);
            c2 = take(m);
            bwd_->push_back({CK_SAVE_WORK, m, c2});
        }
        rev(m, e, c2, S - 1, spine);
        give(c2);
        rev(a, m, c, S, false);
    }
};

inline CkSchedule ck_schedule(int nseg, int slots) { return CkBuilder(nseg, slots).build(); }

}  // namespace psv
