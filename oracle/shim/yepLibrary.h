/* oracle/shim/yepLibrary.h -- the part of the Yeppp! 1.0 C API that the
 * reference followup program calls (followup.c:56-58, 436-447, 467-470),
 * backed by the C library (test infrastructure only; the prebuilt Yeppp!
 * library is not used). */
#ifndef PA_YEP_SHIM_H
#define PA_YEP_SHIM_H
#include <stdbool.h> /* the Yeppp! headers bring in bool/true/false */
#include <stddef.h>
typedef double Yep64f;
typedef size_t YepSize;
enum YepStatus { YepStatusOk = 0, YepStatusNullPointer = 1 };
enum YepStatus yepLibrary_Init(void);
enum YepStatus yepLibrary_Release(void);
enum YepStatus yepMath_Cos_V64f_V64f(const Yep64f *x, Yep64f *y, YepSize n);
enum YepStatus yepMath_Sin_V64f_V64f(const Yep64f *x, Yep64f *y, YepSize n);
#endif
