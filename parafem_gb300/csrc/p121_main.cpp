// p121_main.cpp -- the p121 program (src/programs/5th_ed/p121/p121.f90) with
// its solve on the GPU:  p121 <job> [mode] [device]
//   mode 0: FP64 PCG with checon_par (the p121 drop-in, default)
//   mode 1: FP64 PCG to a relative residual of tol
//   mode 2: FP32-storkm PCG with FP64 defect correction to a relative residual of tol
#include "pfgpu.h"

#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <job> [mode] [device]\n", argv[0]);
        return 1;
    }
    const int mode = argc > 2 ? atoi(argv[2]) : PF_MODE_P121;
    const int device = argc > 3 ? atoi(argv[3]) : 0;
    int iters = 0;
    double central = 0.0;
    if (pf_p121_run(argv[1], &device, &mode, &iters, &central) != PF_SUCCESS) {
        char msg[1024];
        const int len = sizeof msg;
        pf_last_error(msg, &len);
        fprintf(stderr, "p121: %s\n", msg);
        return 1;
    }
    printf("p121: %d iterations, central displacement %.6e\n", iters, central);
    return 0;
}
