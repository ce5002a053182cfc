// p123_main.cpp -- the p123 program (src/programs/5th_ed/p123/p123.f90,
// 3-D Laplace with 8-node bricks) with its solve on the GPU:
//   p123 <job> [device]
// Reads job.dat/.d/.bnd/.lds (and .fix when the deck has fixed freedoms),
// writes job.res and job.ensi.NDPTL-000001.
#include "pfgpu.h"

#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <job> [device]\n", argv[0]);
        return 1;
    }
    const int device = argc > 2 ? atoi(argv[2]) : 0;
    int iters = 0;
    double pot[4] = {0, 0, 0, 0};
    if (pf_p123_run(argv[1], &device, &iters, pot) != PF_SUCCESS) {
        char msg[1024];
        const int len = sizeof msg;
        pf_last_error(msg, &len);
        fprintf(stderr, "p123: %s\n", msg);
        return 1;
    }
    printf("p123: %d iterations, potentials %.4e %.4e %.4e %.4e\n", iters, pot[0], pot[1], pot[2], pot[3]);
    return 0;
}
