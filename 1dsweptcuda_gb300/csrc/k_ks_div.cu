// KS kernels of the DIVISE build (SW_FLAG_KS_DIVIDE, KS1D_SweptShared.cu:111-132):
// the KS translation unit compiled again with the right-hand side dividing by
// 4dx, dx^2 and dx^4, its instances in the namespace sw::ks_divide.
#define SW_KS_DIVIDE_TU 1
#include "k_ks.cu"
