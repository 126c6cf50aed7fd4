// evr_kern_items_d0.cu -- the general term kernel in double, G(Q) from a table or the constant G0.
#define EVR_KT double
#define EVR_KGFLY false
#define EVR_KSLAB 0
#include "evr_kern_inst.cuh"
