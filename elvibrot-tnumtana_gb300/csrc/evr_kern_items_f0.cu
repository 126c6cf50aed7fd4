// evr_kern_items_f0.cu -- the general term kernel in float, G(Q) from a table or the constant G0.
#define EVR_KT float
#define EVR_KGFLY false
#define EVR_KSLAB 0
#include "evr_kern_inst.cuh"
