/* Test-infrastructure shim (oracle build only).
 *
 * cfitsio is not installed in this image.  lyspeq's per-chunk path reads its
 * S/Q lookup tables from FITS image HDUs (io/sq_lookup_table_file.cpp); this
 * header declares the cfitsio calls lyspeq's sources use, with cfitsio's
 * signatures, and minifits.cpp implements the image-HDU subset (create, write
 * keys and double images, open, move by EXTNAME, read keys and images).
 * Binary-table calls (picca spectra, bootstrap files) are declared so those
 * translation units compile; they return a nonzero status.
 */
#ifndef LQG_ORACLE_SHIM_FITSIO_H
#define LQG_ORACLE_SHIM_FITSIO_H

typedef long long LONGLONG;
typedef struct lqg_minifits fitsfile;

#define READONLY 0
#define READWRITE 1
#define IMAGE_HDU 0
#define ASCII_TBL 1
#define BINARY_TBL 2
#define ANY_HDU -1
#define DOUBLE_IMG -64
#define FLOAT_IMG -32
#define TBIT 1
#define TBYTE 11
#define TLOGICAL 14
#define TSTRING 16
#define TSHORT 21
#define TUINT 30
#define TINT 31
#define TULONG 40
#define TLONG 41
#define TFLOAT 42
#define TLONGLONG 81
#define TDOUBLE 82
#define CASESEN 1
#define CASEINSEN 0
#define FLEN_FILENAME 1025
#define FLEN_KEYWORD 75
#define FLEN_CARD 81
#define FLEN_VALUE 71
#define FLEN_COMMENT 73
#define FLEN_ERRMSG 81
#define FLEN_STATUS 31

int fits_open_file(fitsfile **fptr, const char *filename, int iomode, int *status);
int fits_create_file(fitsfile **fptr, const char *filename, int *status);
int fits_close_file(fitsfile *fptr, int *status);
void fits_get_errstatus(int status, char *err_text);
int fits_movnam_hdu(fitsfile *fptr, int hdutype, char *extname, int extver, int *status);
int fits_movabs_hdu(fitsfile *fptr, int hdunum, int *hdutype, int *status);
int fits_get_num_hdus(fitsfile *fptr, int *hdunum, int *status);
int fits_get_hdu_num(fitsfile *fptr, int *hdunum);
int fits_get_hdrspace(fitsfile *fptr, int *keysexist, int *morekeys, int *status);
int fits_read_key(fitsfile *fptr, int datatype, const char *keyname, void *value,
                  char *comm, int *status);
int fits_read_keyn(fitsfile *fptr, int keynum, char *keyname, char *value, char *comm,
                   int *status);
int fits_read_keys_lng(fitsfile *fptr, const char *keyname, int nstart, int nmax,
                       long *value, int *nfound, int *status);
int fits_make_keyn(const char *keyroot, int value, char *keyname, int *status);
int fits_get_num_cols(fitsfile *fptr, int *ncols, int *status);
int fits_get_num_rows(fitsfile *fptr, long *nrows, int *status);
int fits_get_colnum(fitsfile *fptr, int casesen, char *templt, int *colnum, int *status);
int fits_read_col(fitsfile *fptr, int datatype, int colnum, LONGLONG firstrow,
                  LONGLONG firstelem, LONGLONG nelem, void *nulval, void *array,
                  int *anynul, int *status);
int fits_read_tdim(fitsfile *fptr, int colnum, int maxdim, int *naxis, long *naxes,
                   int *status);
int fits_create_img(fitsfile *fptr, int bitpix, int naxis, long *naxes, int *status);
int fits_write_img(fitsfile *fptr, int datatype, LONGLONG firstelem, LONGLONG nelem,
                   void *array, int *status);
int fits_read_img(fitsfile *fptr, int datatype, LONGLONG firstelem, LONGLONG nelem,
                  void *nulval, void *array, int *anynul, int *status);
int fits_write_key(fitsfile *fptr, int datatype, const char *keyname, void *value,
                   const char *comment, int *status);
int fits_update_key_str(fitsfile *fptr, const char *keyname, const char *value,
                        const char *comment, int *status);
int fits_write_comment(fitsfile *fptr, const char *comment, int *status);

#endif
