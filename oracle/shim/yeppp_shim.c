/* oracle/shim/yeppp_shim.c -- element-wise cos/sin with the C library for
 * the Yeppp! calls of the reference followup program (test infrastructure
 * only). */
#include <math.h>
#include "yepLibrary.h"

/* number of vector cos calls (one per detector per Fstatnet evaluation);
 * read by the reference-followup driver to count evaluations */
long pa_yep_cos_calls = 0;

enum YepStatus yepLibrary_Init(void) { return YepStatusOk; }
enum YepStatus yepLibrary_Release(void) { return YepStatusOk; }

enum YepStatus yepMath_Cos_V64f_V64f(const Yep64f *x, Yep64f *y, YepSize n) {
  if (!x || !y) return YepStatusNullPointer;
  pa_yep_cos_calls++;
  for (YepSize i = 0; i < n; i++) y[i] = cos(x[i]);
  return YepStatusOk;
}

enum YepStatus yepMath_Sin_V64f_V64f(const Yep64f *x, Yep64f *y, YepSize n) {
  if (!x || !y) return YepStatusNullPointer;
  for (YepSize i = 0; i < n; i++) y[i] = sin(x[i]);
  return YepStatusOk;
}
