/* Minimal stand-in for the configure-generated config.h of GSL 2.4, enough to
 * compile the handful of GSL sources the oracle cross-check links (Bessel I0,
 * subset index sort, hypot, integer powers, error handling) on glibc. */
#define HAVE_DECL_HYPOT 1
#define HAVE_DECL_LOG1P 1
#define HAVE_DECL_EXPM1 1
#define HAVE_DECL_ACOSH 1
#define HAVE_DECL_ASINH 1
#define HAVE_DECL_ATANH 1
#define HAVE_DECL_LDEXP 1
#define HAVE_DECL_FREXP 1
#define HAVE_DECL_ISINF 1
#define HAVE_DECL_ISFINITE 1
#define HAVE_DECL_FINITE 1
#define HAVE_DECL_ISNAN 1
#define HAVE_EXIT_SUCCESS_AND_FAILURE 1
#define HAVE_IEEE_COMPARISONS 1
#define HAVE_IEEE_DENORMALS 1
#define GSL_COERCE_DBL(x) (x)
#define DISCARD_POINTER(p) do { ; } while(p ? 0 : 0);
#define GSL_RANGE_CHECK 0
#define RETURN_IF_NULL(x) if (!x) { return ; }
