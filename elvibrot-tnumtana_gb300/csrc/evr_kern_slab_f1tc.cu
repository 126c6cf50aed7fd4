// evr_kern_slab_f1tc.cu -- the slab-streaming term kernel in float with tensor-core contractions, G(Q) from the linear model per point.
#define EVR_KT float
#define EVR_KGFLY true
#define EVR_KSLAB 1
#define EVR_KTC true
#include "evr_kern_inst.cuh"
