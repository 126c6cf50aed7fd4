// evr_kern_slab_f0tc.cu -- the slab-streaming term kernel in float with tensor-core contractions, G(Q) from a table or the constant G0.
#define EVR_KT float
#define EVR_KGFLY false
#define EVR_KSLAB 1
#define EVR_KTC true
#include "evr_kern_inst.cuh"
