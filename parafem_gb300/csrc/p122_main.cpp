// p122_main.cpp -- the p122 program (src/programs/5th_ed/p122/p122.f90,
// Mohr-Coulomb viscoplasticity with 20-node bricks under load control) with
// its solves on the GPU:  p122 <job> [device]
// Reads job.dat/.d/.bnd/.lds, writes job.res and job.ensi.DISPL-0000nn.
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
    int incs = 0;
    if (pf_p122_run(argv[1], &device, &incs) != PF_SUCCESS) {
        char msg[1024];
        const int len = sizeof msg;
        pf_last_error(msg, &len);
        fprintf(stderr, "p122: %s\n", msg);
        return 1;
    }
    printf("p122: %d load increments\n", incs);
    return 0;
}
