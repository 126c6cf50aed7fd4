// evr_kern_slab_f1.cu -- the slab-streaming term kernel in float, G(Q) from the linear model per point.
#define EVR_KT float
#define EVR_KGFLY true
#define EVR_KSLAB 1
#include "evr_kern_inst.cuh"
