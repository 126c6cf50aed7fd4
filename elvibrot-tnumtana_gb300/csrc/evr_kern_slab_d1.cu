// evr_kern_slab_d1.cu -- the slab-streaming term kernel in double, G(Q) from the linear model per point.
#define EVR_KT double
#define EVR_KGFLY true
#define EVR_KSLAB 1
#include "evr_kern_inst.cuh"
