// evr_kern_slab_d0.cu -- the slab-streaming term kernel in double, G(Q) from a table or the constant G0.
#define EVR_KT double
#define EVR_KGFLY false
#define EVR_KSLAB 1
#include "evr_kern_inst.cuh"
