/* Forwards the LAPACK symbol the reference header declares (dsyev_,
 * framework/hp_numeric.h:500-520) to the copy exported by the OpenBLAS that
 * scipy bundles in this container.  Oracle build only. */
extern void scipy_dsyev_(char *, char *, int *, double *, int *, double *, double *, int *, int *);
void dsyev_(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work, int *lwork, int *info) {
  scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info);
}
