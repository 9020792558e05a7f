/* shim: only the names the reference's headers mention */
#include "shim.h"
#ifndef REF_SHIM_CURAND
#define REF_SHIM_CURAND
#define CURAND_PI_DOUBLE (3.1415926535897932)
#define CURAND_2PI (6.2831855f) /* a float constant, as in the CUDA toolkit */
struct curandStateXORWOW { unsigned int d, v[5]; int boxmuller_flag; int boxmuller_flag_double; float boxmuller_extra; double boxmuller_extra_double; };
typedef struct curandStateXORWOW curandState;
#endif
