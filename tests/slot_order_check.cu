// Host check of the panel sweeps' target order (BsJob::slots, bs_slot_target in
// sb_kernels.h): reads "M n_wings points_0 ... points_{n-1}" lines from stdin and prints, per
// line, the target index of every slot (rows of sum(points) points, wings in order).
#include <cstdio>
#include <vector>

#include "sb_kernels.h"

int main() {
    long long M;
    int S;
    while (std::scanf("%lld %d", &M, &S) == 2) {
        sbgpu::BsJob J;
        std::vector<int> pts(S);
        int Np = 0;
        for (int w = 0; w < S; ++w) {
            std::scanf("%d", &pts[w]);
            J.group_off[w] = Np;
            Np += pts[w];
        }
        J.group_off[S] = Np;
        J.M = M;
        J.row_pts = Np;
        J.n_groups = S;
        J.slots = (M + Np - 1) / Np * Np;
        for (long long s = 0; s < J.slots; ++s) std::printf("%lld ", sbgpu::bs_slot_target(J, s));
        std::printf("\n");
    }
    return 0;
}
