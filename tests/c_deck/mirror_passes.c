/* White-box check of the drop-in's host passes over the mirrors: the
 * threaded compare (mirror_differs) and copy (mirror_copy) of em2d_host.c,
 * on spans around the 4 MB split and with one flipped byte at the ends and
 * in the middle.  No CUDA call is made.  Prints "ok" and returns 0. */
#include "../../zpic_gb300/csrc/em2d/em2d_host.c"

int main(void)
{
    const size_t mb4 = (size_t)4 << 20;
    const size_t sizes[] = {0, 1, 7, mb4 - 1, mb4, mb4 + 3, 9 * mb4 + 11, 50 * mb4};
    for (unsigned s = 0; s < sizeof(sizes) / sizeof(sizes[0]); s++) {
        const size_t n = sizes[s];
        unsigned char *a = (unsigned char *)malloc(n + 1), *b = (unsigned char *)malloc(n + 1);
        if (!a || !b) return 2;
        for (size_t i = 0; i < n; i++) a[i] = (unsigned char)((i * 2654435761u) >> 13);
        memset(b, 0xAB, n + 1);
        mirror_copy(b, a, n);
        if (memcmp(a, b, n) != 0 || b[n] != 0xAB) {
            printf("copy failed at %zu bytes\n", n);
            return 1;
        }
        if (mirror_differs(a, b, n)) {
            printf("equal spans reported different at %zu bytes\n", n);
            return 1;
        }
        if (n > 0) {
            const size_t pos[] = {0, n / 3, n / 2, n - 1};
            for (int p = 0; p < 4; p++) {
                b[pos[p]] ^= 1;
                if (!mirror_differs(a, b, n)) {
                    printf("a flipped byte at %zu of %zu went unseen\n", pos[p], n);
                    return 1;
                }
                b[pos[p]] ^= 1;
            }
        }
        free(a);
        free(b);
    }
    printf("ok\n");
    return 0;
}
