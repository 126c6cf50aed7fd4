// evr_kern_items_d1.cu -- the general term kernel in double, G(Q) from the linear model per point.
#define EVR_KT double
#define EVR_KGFLY true
#define EVR_KSLAB 0
#include "evr_kern_inst.cuh"
