/* TEST INFRASTRUCTURE ONLY: forced-include for compiling KINC's Pairwise::
 * sources.  The real ExpressionMatrix is an ACE data object; the models only
 * ask it for the sample count. */
#ifndef KINC_REF_SHIM_PRE_H
#define KINC_REF_SHIM_PRE_H
struct ExpressionMatrix
{
   int sampleSize;
   int getSampleSize() const { return sampleSize; }
};
#endif
