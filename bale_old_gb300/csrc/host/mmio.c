/* mmio.c -- MatrixMarket files and binary sparse matrix datasets of the
 * reference's kinds: the host side.
 *
 * spmat's write_matrix_mm (spmat/spmat_utils.upc:128-149) writes
 *   %%MatrixMarket matrix coordinate pattern
 *   <numrows> <numcols> <nnz>
 *   <row+1> <col+1>            (one line per nonzero, rows in order)
 * and read_matrix_mm_to_dist (:217-370) reads "coordinate" files whose field
 * is "pattern" or "integer" (the value is ignored), 1-based, keeping the file
 * order of the nonzeros within each row.  The body is parsed on the device
 * (spmat_io.cu); here are the writers and the header readers.
 */
#include <ctype.h>
#include <inttypes.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include "bale_gb300.h"

int bale_write_matrix_mm(const sparsemat_t *A, const char *path) {
  if (!A || !path || A->numrows < 0 || (A->numrows > 0 && !A->loffset)) return BALE_EINVAL;
  FILE *fp = fopen(path, "w");
  if (!fp) return BALE_EINPUT;
  int ok = fprintf(fp, "%%%%MatrixMarket matrix coordinate pattern\n") > 0;
  ok = ok && fprintf(fp, "%" PRId64 " %" PRId64 " %" PRId64 "\n", A->numrows, A->numcols, A->nnz) > 0;
  for (int64_t i = 0; ok && i < A->numrows; i++)
    for (int64_t j = A->loffset[i]; ok && j < A->loffset[i + 1]; j++)
      ok = fprintf(fp, "%" PRId64 " %" PRId64 "\n", i + 1, A->lnonzero[j] + 1) > 0;
  if (fclose(fp) != 0) ok = 0;
  return ok ? BALE_OK : BALE_EINPUT;
}

/* The banner (object, format, field), comment lines starting with '%', and
 * the size line.  *body receives the byte offset where the entries start;
 * *fields is 2 for pattern files, 3 for integer ones. */
int bale_mm_header(const char *path, int64_t *numrows, int64_t *numcols, int64_t *nnz, int64_t *body,
                   int *fields) {
  if (!path || !numrows || !numcols || !nnz || !body || !fields) return BALE_EINVAL;
  FILE *fp = fopen(path, "r");
  if (!fp) return BALE_EINPUT;
  char line[1024], object[64], format[64], field[64];
  int rc = BALE_EINPUT;
  if (!fgets(line, sizeof line, fp)) goto done;
  if (sscanf(line, "%%%%MatrixMarket %63s %63s %63s", object, format, field) != 3) goto done;
  for (char *c = object; *c; c++) *c = (char)tolower((unsigned char)*c);
  for (char *c = format; *c; c++) *c = (char)tolower((unsigned char)*c);
  for (char *c = field; *c; c++) *c = (char)tolower((unsigned char)*c);
  if (strcmp(object, "matrix") || strcmp(format, "coordinate")) goto done;
  if (!strcmp(field, "pattern")) *fields = 2;
  else if (!strcmp(field, "integer")) *fields = 3;
  else goto done;
  for (;;) {
    if (!fgets(line, sizeof line, fp)) goto done;
    if (line[0] != '%') break;
  }
  if (sscanf(line, "%" SCNd64 " %" SCNd64 " %" SCNd64, numrows, numcols, nnz) != 3 || *numrows < 0 ||
      *numcols < 0 || *nnz < 0)
    goto done;
  *body = (int64_t)ftell(fp);
  rc = BALE_OK;
done:
  fclose(fp);
  return rc;
}

/* Binary datasets (spmat/spmat_agi.upc:245-335 write_rowcounts and
 * write_sparse_matrix_agi, spmat/spmat_exstack.upc:494-686
 * write_sparse_matrix_exstack, spmat/spmat_utils.upc:159-206 the metadata
 * file): a directory holding "metadata" (numrows, numcols, nnz and the
 * number of writers, one decimal per line), and per writer w "rowcnt_<w>"
 * (its rows' lengths) and "nonzero_<w>" (their columns, row after row), both
 * raw int64.  Writer w of W takes the w-th block of (numrows + W - w - 1) / W
 * consecutive rows.  This writes the one-writer dataset the reference writes
 * at one PE. */
int bale_write_sparse_matrix(const char *dirname, const sparsemat_t *A) {
  if (!dirname || !A || A->numrows < 0 || !A->loffset || (A->nnz > 0 && !A->lnonzero)) return BALE_EINVAL;
  char name[4096];
  mkdir(dirname, 0770);  /* may exist already, as in the reference */
  if (snprintf(name, sizeof name, "%s/metadata", dirname) >= (int)sizeof name) return BALE_EINVAL;
  FILE *fp = fopen(name, "w");
  if (!fp) return BALE_EINPUT;
  int ok = fprintf(fp, "%" PRId64 "\n%" PRId64 "\n%" PRId64 "\n%d\n", A->numrows, A->numcols, A->nnz, 1) > 0;
  if (fclose(fp) != 0) ok = 0;
  snprintf(name, sizeof name, "%s/rowcnt_0", dirname);
  if (!ok || !(fp = fopen(name, "wb"))) return BALE_EINPUT;
  for (int64_t i = 0; ok && i < A->numrows; i++) {
    const int64_t rc = A->loffset[i + 1] - A->loffset[i];
    ok = fwrite(&rc, sizeof rc, 1, fp) == 1;
  }
  if (fclose(fp) != 0) ok = 0;
  snprintf(name, sizeof name, "%s/nonzero_0", dirname);
  if (!ok || !(fp = fopen(name, "wb"))) return BALE_EINPUT;
  const size_t nnz = (size_t)(A->numrows > 0 ? A->loffset[A->numrows] : 0);
  ok = nnz == 0 || fwrite(A->lnonzero, sizeof(int64_t), nnz, fp) == nnz;
  if (fclose(fp) != 0) ok = 0;
  return ok ? BALE_OK : BALE_EINPUT;
}

/* The metadata file, read as read_sparse_matrix_metadata does (four "%ld"). */
int bale_sparse_matrix_header(const char *dirname, int64_t *numrows, int64_t *numcols, int64_t *nnz,
                              int64_t *nwriters) {
  if (!dirname || !numrows || !numcols || !nnz || !nwriters) return BALE_EINVAL;
  char name[4096];
  if (snprintf(name, sizeof name, "%s/metadata", dirname) >= (int)sizeof name) return BALE_EINVAL;
  FILE *fp = fopen(name, "r");
  if (!fp) return BALE_EINPUT;
  const int got = fscanf(fp, "%" SCNd64 " %" SCNd64 " %" SCNd64 " %" SCNd64, numrows, numcols, nnz, nwriters);
  fclose(fp);
  if (got != 4 || *numrows < 0 || *numcols < 0 || *nnz < 0 || *nwriters < 1) return BALE_EINPUT;
  return BALE_OK;
}
