/* The r^2.5 algorithm of the FP64 kernels (pow25_core in
 * allscale_ipic3d_gb300/csrc/particle_kernels.cuh), run on the host in C
 * with fma(), for a test against correctly rounded values. The reciprocal
 * square root the device takes from rsqrt() (error <= 1 ulp) is replaced by
 * the correctly rounded 1/sqrt(a) and by its two neighbours, so that every
 * value the device function may return for it is covered.
 * Reads doubles from the file argv[1]; writes 3 doubles per input to stdout. */
#include <math.h>
#include <stdio.h>

static double core(double a, double y) {
    double s = a * y;
    double e = fma(-s, s, a);
    s = s + (e * y) * 0.5;
    e = fma(-s, s, a);
    const double ds = (e * y) * 0.5;
    const double p = a * a, pe = fma(a, a, -p);
    const double h = p * s;
    double l = fma(p, s, -h);
    l = l + (p * ds + pe * s);
    return h + l;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    double a;
    while (fread(&a, sizeof a, 1, f) == 1) {
        const double y = (double)(1.0L / sqrtl((long double)a));
        const double out[3] = {core(a, nextafter(y, 0.0)), core(a, y), core(a, nextafter(y, INFINITY))};
        fwrite(out, sizeof(double), 3, stdout);
    }
    fclose(f);
    return 0;
}
