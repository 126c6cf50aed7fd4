// evr_kern_slab_f0.cu -- the slab-streaming term kernel in float, G(Q) from a table or the constant G0.
#define EVR_KT float
#define EVR_KGFLY false
#define EVR_KSLAB 1
#include "evr_kern_inst.cuh"
