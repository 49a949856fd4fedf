/*
 * lapack_shim.c -- LAPACK entry points for the reference build in oracle/_ref.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference links an unpinned system -llapack
 * (lib/makefile, main/dmrg/xxz_vf/makefile:17,22); none is installed here, so the four
 * routines it calls are forwarded to the LAPACK bundled with scipy (exported there with a
 * "scipy_" prefix).  Only used to build the reference for validating the oracle.
 */
extern void scipy_dstev_(char *, int *, double *, double *, double *, int *, double *, int *);
extern void scipy_dsyev_(const char *, const char *, const int *, double *, const int *, double *, double *, const int *, int *);
extern void scipy_dgeev_(const char *, const char *, const int *, double *, const int *, double *, double *, double *,
                         const int *, double *, const int *, double *, const int *, int *);
extern void scipy_dgesvd_(const char *, const char *, const int *, const int *, double *, const int *, double *, double *,
                          const int *, double *, const int *, double *, const int *, int *);

void dstev_(char *jobz, int *n, double *d, double *e, double *z, int *ldz, double *work, int *info) {
   scipy_dstev_(jobz, n, d, e, z, ldz, work, info);
}

void dsyev_(const char *jobz, const char *uplo, const int *n, double *a, const int *lda, double *w, double *work, const int *lwork,
            int *info) {
   scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info);
}

void dgeev_(const char *jobvl, const char *jobvr, const int *n, double *a, const int *lda, double *wr, double *wi, double *vl,
            const int *ldvl, double *vr, const int *ldvr, double *work, const int *lwork, int *info) {
   scipy_dgeev_(jobvl, jobvr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork, info);
}

void dgesvd_(const char *jobu, const char *jobvt, const int *m, const int *n, double *a, const int *lda, double *s, double *u,
             const int *ldu, double *vt, const int *ldvt, double *work, const int *lwork, int *info) {
   scipy_dgesvd_(jobu, jobvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, info);
}

extern void scipy_dspgv_(const int *, const char *, const char *, const int *, double *, double *, double *, double *,
                         const int *, double *, int *);

void dspgv_(const int *itype, const char *jobz, const char *uplo, const int *n, double *ap, double *bp, double *w, double *z,
            const int *ldz, double *work, int *info) {
   scipy_dspgv_(itype, jobz, uplo, n, ap, bp, w, z, ldz, work, info);
}
