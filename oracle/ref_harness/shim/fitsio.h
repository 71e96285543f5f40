/* stand-in for cfitsio: only the names the reference's headers mention */
#pragma once
typedef struct fitsfile fitsfile;
int fits_open_file(fitsfile**, const char*, int, int*);
int fits_close_file(fitsfile*, int*);
void fits_report_error(void*, int);
