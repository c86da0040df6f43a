/*
 * Used only by the FP64-promoted oracle build (reference compiled with
 * -Dfloat=double).  The reference's input_float / input_float_vector
 * (Parsing.c:459-527, 701-745) scan "%f" into what that build turns into a
 * double, which stores garbage.  That build compiles Parsing.c with those two
 * names renamed away and links these replacements, which forward to the
 * reference's own input_double / input_double_vector (same default/range
 * handling, "%lf" scanning).
 */
int input_double(char *, double *, char *, int);
int input_double_vector(char *, int, double *, int);

int input_float(char *name, double *value, char *interpret, int m)
{
	return input_double(name, value, interpret, m);
}

int input_float_vector(char *name, int number, double *value, int m)
{
	return input_double_vector(name, number, value, m);
}
