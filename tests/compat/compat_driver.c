/*
 * compat_driver.c -- TEST INFRASTRUCTURE: one steered frame through the
 * reference's own function names (include/ivr_compat.h), in the order of the
 * reference's server (main.c:145-168 start-up, main.c:226-248 frame), with
 * every brick's sub-image, the composited frame and its RGBA8 written out.
 *
 *   compat_driver vol.raw w h d dataendian colormap xfer rows cols slabs
 *                 tilew tileh state.bin lut.bin|- lutoffset outprefix
 *
 * Writes <outprefix>.bricks (K sub-images, RGBA32), <outprefix>.frame
 * (RGBA32), <outprefix>.rgba8 and <outprefix>.info ("vw vh K").  Exit 0 on
 * success; otherwise the layer's message on stderr.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ivr_compat.h"

static int check(const char *where)
{
    const char *e = ivr_compat_last_error();
    if (e && e[0]) {
        fprintf(stderr, "%s: %s\n", where, e);
        return 1;
    }
    return 0;
}

static int dump(const char *prefix, const char *ext, const void *p, size_t n, const char *mode)
{
    char path[1024];
    snprintf(path, sizeof path, "%s.%s", prefix, ext);
    FILE *f = fopen(path, mode);
    if (!f) return 1;
    int bad = fwrite(p, 1, n, f) != n;
    return fclose(f) != 0 || bad;
}

int main(int argc, char **argv)
{
    if (argc != 17) {
        fprintf(stderr, "usage: %s vol w h d dataendian colormap xfer rows cols slabs tilew tileh state lut|- "
                        "lutoffset outprefix\n", argv[0]);
        return 2;
    }
    ivr_cmdargs args;
    memset(&args, 0, sizeof args);
    strncpy(args.filename, argv[1], sizeof args.filename - 1);
    args.width = atoi(argv[2]);
    args.height = atoi(argv[3]);
    args.depth = atoi(argv[4]);
    args.dataendian = atoi(argv[5]);
    args.colormap = atoi(argv[6]);
    args.xfer = atoi(argv[7]);
    for (int i = 0; i < 3; i++) args.procdims[i] = atoi(argv[8 + i]);
    args.tilewid = atoi(argv[11]);
    args.tilehgt = atoi(argv[12]);
    const char *prefix = argv[16];

    /* the steering message, as recvstate() delivers it (main.c:209-213) */
    FILE *fs = fopen(argv[13], "rb");
    if (!fs || fread(&mystate, 1, sizeof mystate, fs) != sizeof mystate) return 3;
    fclose(fs);
    winwidth = mystate.winwidth;
    winheight = mystate.winheight;

    if (init(args, 0) != 0) {
        check("init");
        return 1;
    }
    if (args.colormap == -1) {  /* a LUT set directly (main.c:64-65,80) */
        FILE *fl = fopen(argv[14], "rb");
        if (!fl) return 4;
        fseek(fl, 0, SEEK_END);
        long bytes = ftell(fl);
        fseek(fl, 0, SEEK_SET);
        lut = (ivr_color4f *) malloc((size_t) bytes);
        if (!lut || fread(lut, 1, (size_t) bytes, fl) != (size_t) bytes) return 4;
        fclose(fl);
        lutoffset = atoi(argv[15]);
        maxlutindx = (int) (bytes / (long) sizeof(ivr_color4f)) - 1;
    }

    /* main.c:226-233 */
    float planeconst[6] = {pzero[0], pzero[1], pzero[2], pzero[3], pzero[4], pzero[5]};
    setviewport(&viewport, 0, 0, winwidth, winheight);
    setplaneconst(planeconst, mystate.newconst);
    setmvm(mvm, mystate.mvm);
    setpm(pm, mystate.pm);
    setfrustum(&viewvolume, mystate.vv);
    updatevolbbox();
    initcolbufs(0);
    if (check("frame set-up")) return 1;

    const int K = args.procdims[0] * args.procdims[1] * args.procdims[2];
    const size_t npix = (size_t) viewport.w * (size_t) viewport.h;
    for (int r = 0; r < K; r++) {  /* every rank's createlocalimage (main.c:238) */
        createlocalimage(r);
        if (check("createlocalimage")) return 1;
        if (dump(prefix, "bricks", colorbuf, npix * sizeof(ivr_color4f), r ? "ab" : "wb")) return 5;
    }
    if (compositelocalimage() != 0) {  /* main.c:241 */
        check("compositelocalimage");
        return 1;
    }
    if (dump(prefix, "frame", colorbuf, npix * sizeof(ivr_color4f), "wb")) return 5;
    if (writetomemory(0, 0) != 0) {
        check("writetomemory");
        return 1;
    }
    if (dump(prefix, "rgba8", tiffimage, npix * 4, "wb")) return 5;

    char info[64];
    int n = snprintf(info, sizeof info, "%d %d %d\n", (int) viewport.w, (int) viewport.h, K);
    if (dump(prefix, "info", info, (size_t) n, "wb")) return 5;
    freeall();
    return 0;
}
