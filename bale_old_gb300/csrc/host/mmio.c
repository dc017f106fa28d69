/* mmio.c -- MatrixMarket files of the reference's kind: the host side.
 *
 * spmat's write_matrix_mm (spmat/spmat_utils.upc:128-149) writes
 *   %%MatrixMarket matrix coordinate pattern
 *   <numrows> <numcols> <nnz>
 *   <row+1> <col+1>            (one line per nonzero, rows in order)
 * and read_matrix_mm_to_dist (:217-370) reads "coordinate" files whose field
 * is "pattern" or "integer" (the value is ignored), 1-based, keeping the file
 * order of the nonzeros within each row.  The body is parsed on the device
 * (graph.cu); here are the writer and the header reader.
 */
#include <ctype.h>
#include <inttypes.h>
#include <stdio.h>
#include <string.h>

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
