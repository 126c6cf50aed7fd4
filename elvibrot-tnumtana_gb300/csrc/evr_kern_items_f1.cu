// evr_kern_items_f1.cu -- the general term kernel in float, G(Q) from the linear model per point.
#define EVR_KT float
#define EVR_KGFLY true
#define EVR_KSLAB 0
#include "evr_kern_inst.cuh"
