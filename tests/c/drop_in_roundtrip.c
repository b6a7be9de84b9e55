/*
 * A C caller of the drop-in API, written the way libdwt's users call it:
 * host image from dwt_util_alloc_image at the "optimal" prime row stride,
 * the test pattern, a full forward CDF 9/7 decomposition, the HH1 subband
 * located with dwt_util_subband_s, the log-magnitude view saved as PGM, the
 * inverse, and the round trip checked with dwt_util_compare_s.  The same
 * sequence then runs with CDF 5/3.  Exit status 0 on success.
 *
 * usage: drop_in_roundtrip <size_x> <size_y> <output.pgm>
 */
#include <stdio.h>
#include <stdlib.h>

#include "libdwt.h"

static int run(int x, int y, const char *pgm, int wavelet97)
{
    const int stride_x = dwt_util_get_opt_stride(x * (int)sizeof(float));
    const int stride_y = sizeof(float);
    void *img = NULL, *ref = NULL, *view = NULL;
    dwt_util_alloc_image(&img, stride_x, stride_y, x, y);
    dwt_util_alloc_image(&ref, stride_x, stride_y, x, y);
    dwt_util_alloc_image(&view, stride_x, stride_y, x, y);
    dwt_util_test_image_fill_s(img, stride_x, stride_y, x, y, 0);
    dwt_util_test_image_fill_s(ref, stride_x, stride_y, x, y, 0);

    int j = -1;
    if (wavelet97)
        dwt_cdf97_2f_s(img, stride_x, stride_y, x, y, x, y, &j, 0, 0);
    else
        dwt_cdf53_2f_s(img, stride_x, stride_y, x, y, x, y, &j, 0, 0);
    if (j < 1) {
        dwt_util_log(LOG_ERR, "no decomposition (j = %d)\n", j);
        return 1;
    }

    void *hh = NULL;
    int hx = 0, hy = 0;
    dwt_util_subband_s(img, stride_x, stride_y, x, y, x, y, 1, DWT_HH, &hh, &hx, &hy);
    if (hx != x / 2 || hy != y / 2 || (char *)hh != (char *)img + (y + 1) / 2 * stride_x + (x + 1) / 2 * stride_y) {
        dwt_util_log(LOG_ERR, "HH1 subband at the wrong place\n");
        return 1;
    }
    dwt_util_conv_show_s(img, view, stride_x, stride_y, x, y);
    if (pgm && dwt_util_save_to_pgm_s(pgm, 1.0f, view, stride_x, stride_y, x, y)) return 1;

    if (wavelet97)
        dwt_cdf97_2i_s(img, stride_x, stride_y, x, y, x, y, j, 0, 0);
    else
        dwt_cdf53_2i_s(img, stride_x, stride_y, x, y, x, y, j, 0, 0);
    const int bad = dwt_util_compare_s(img, ref, stride_x, stride_y, x, y);
    dwt_util_log(bad ? LOG_ERR : LOG_INFO, "%s %dx%d j=%d round trip: %s\n", wavelet97 ? "cdf97" : "cdf53", x, y, j,
                 bad ? "differs" : "ok");
    dwt_util_free_image(&img);
    dwt_util_free_image(&ref);
    dwt_util_free_image(&view);
    return bad;
}

int main(int argc, char *argv[])
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s <size_x> <size_y> <output.pgm>\n", argv[0]);
        return 2;
    }
    dwt_util_init();
    const int x = atoi(argv[1]), y = atoi(argv[2]);
    int bad = run(x, y, argv[3], 1);
    bad |= run(x, y, NULL, 0);
    dwt_util_finish();
    return bad;
}
