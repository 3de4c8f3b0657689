/* Empty stand-in: the reference includes <mpfr.h> but uses none of it on the solve path. */
