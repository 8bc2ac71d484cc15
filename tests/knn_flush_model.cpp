// CPU model of k_knn_t33's per-lane candidate queue and its flush, built from the
// same comparator networks (asg_knn_net.cuh).  For bundles of 32 queries it
// streams every particle as a candidate in a shuffled order, queues the ones at
// or below the lane's current 33rd value, and flushes all 32 queues when any
// holds more than KNN_QUEUE - 2 after a step of two candidates, as the kernel
// does.  The result must be the exact 33rd smallest squared distance, and the
// tie flag must be set whenever more than one particle sits at that distance.
// Points: a lattice with duplicated sites (many exact ties) plus uniform
// points.  Exit status 0 when every query agrees.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#define __device__
#define __forceinline__ inline
#include "../asmooth_gb300/csrc/asg_knn_net.cuh"

using namespace asg;

static float norm2(const float* a, const float* b)
{
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return (dx * dx + dy * dy) + dz * dz;  // built with -ffp-contract=off
}

struct Lane {
    float a[33];
    float q[KNN_QUEUE];
    int qn = 0;
    bool tie = false;
};

static void flush(Lane& L)
{
    float v[KNN_QUEUE];
    for (int i = 0; i < KNN_QUEUE; ++i) v[i] = i < L.qn ? L.q[i] : INFINITY;
    L.qn = 0;
    knn_sort16(v);
    const float old = L.a[32];
    const float t34 = knn_merge33(L.a, v);
    const float top = L.a[32];
    L.tie = (top == old && L.tie) || t34 == top;
}

int main()
{
    std::mt19937 rng(12345);
    std::vector<float> x;
    const int g = 12;
    for (int i = 0; i < g; ++i)
        for (int j = 0; j < g; ++j)
            for (int k = 0; k < g; ++k) {
                const int copies = (i + 2 * j + 3 * k) % 7 == 0 ? 2 : 1;
                for (int c = 0; c < copies; ++c) {
                    x.push_back(0.5f * i);
                    x.push_back(0.5f * j);
                    x.push_back(0.5f * k);
                }
            }
    std::uniform_real_distribution<float> u(0.0f, 0.5f * g);
    for (int i = 0; i < 1500; ++i)
        for (int a = 0; a < 3; ++a) x.push_back(u(rng));
    const int n = (int)x.size() / 3;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    long long bad = 0, ties = 0, flagged = 0;
    for (int base = 0; base < n; base += 32) {
        const int nq = std::min(32, n - base);
        std::vector<Lane> L(nq);
        for (auto& l : L) std::fill(l.a, l.a + 33, INFINITY);
        std::shuffle(order.begin(), order.end(), rng);
        for (int s = 0; s < n; s += 2) {
            bool full = false;
            for (int l = 0; l < nq; ++l) {
                for (int t = s; t < std::min(s + 2, n); ++t) {
                    const float d2 = norm2(&x[3 * (base + l)], &x[3 * order[t]]);
                    if (d2 <= L[l].a[32]) L[l].q[L[l].qn++] = d2;
                }
                full |= L[l].qn > KNN_QUEUE - 2;
            }
            if (full)
                for (auto& l : L) flush(l);
        }
        for (auto& l : L)
            if (l.qn > 0) {
                for (auto& m : L) flush(m);
                break;
            }
        for (int l = 0; l < nq; ++l) {
            std::vector<float> d(n);
            for (int j = 0; j < n; ++j) d[j] = norm2(&x[3 * (base + l)], &x[3 * j]);
            std::sort(d.begin(), d.end());
            const float t33 = d[32];
            const bool truth = d[33] == t33 || d[31] == t33;
            const bool flag = L[l].tie || L[l].a[31] == L[l].a[32];
            ties += truth;
            flagged += flag;
            if (L[l].a[32] != t33 || (truth && !flag)) ++bad;
        }
    }
    std::printf("queries %d exact ties %lld flagged %lld wrong %lld\n", n, ties, flagged, bad);
    return bad == 0 && ties > 0 ? 0 : 1;
}
