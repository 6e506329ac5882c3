/* The reference's cal2DReduction.c calls omp_get_thread_num() outside its
 * _OPENMP guards; built serially (without libgomp) it gets this one-thread
 * answer.  Build shim only: the reference's sources are compiled unmodified. */
int omp_get_thread_num(void)
{
    return 0;
}
