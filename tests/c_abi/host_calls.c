/* A plain C caller of the library's host-only entry points, compiled with a
 * C compiler against include/scir_gb300.h: the header must be valid C and
 * the symbols must link.  Prints one value per line for the Python test. */
#include <stdio.h>

#include "scir_gb300.h"

int main(void) {
    printf("abi %d\n", scir_abi_version());
    printf("ok %s\n", scir_status_string(SCIR_OK));
    printf("valid_len %lld\n", (long long)scir_fir_out_len(65536, 63, SCIR_FIR_VALID));

    int64_t sizes[16];
    int64_t count = 0;
    int rc = scir_host_chunk_plan(1024, (size_t)1 << 20, (size_t)1 << 20, 128, sizes, 16, &count);
    printf("plan %d %lld", rc, (long long)count);
    for (int64_t i = 0; i < count && i < 16; ++i) printf(" %lld", (long long)sizes[i]);
    printf("\n");

    double cut = 0.2, h[63];
    rc = scir_firwin(63, &cut, 1, SCIR_WIN_HAMMING, 0.0, 1, 1, 0.0, h);
    printf("firwin %d", rc);
    for (int i = 0; i < 63; ++i) printf(" %.17g", h[i]);
    printf("\n");

    double wn[2] = {0.001, 0.002}, sos[8 * 6];
    int nsec = 0;
    rc = scir_iirfilter_sos(8, SCIR_IIR_BUTTER, SCIR_BAND_BANDPASS, wn, 0.0, 0.0, sos, 8, &nsec);
    printf("butter %d %d", rc, nsec);
    for (int i = 0; i < nsec * 6; ++i) printf(" %.17g", sos[i]);
    printf("\n");

    /* a bad call reports its status and a message */
    rc = scir_host_chunk_plan(0, 4, 4, 1, NULL, 0, &count);
    char msg[256];
    scir_last_error(msg, sizeof msg);
    printf("bad %d %s\n", rc, msg[0] ? "message" : "none");
    return 0;
}
