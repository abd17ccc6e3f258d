// ivr_frame.h -- host-side frame geometry and LUT builders.
#pragma once

#include "ivr_internal.h"

namespace ivr {

// Brick `rank` of a py x px x pz decomposition (getlocalbrick + the AABB of
// initvolbbox); fills the geometry fields of b.
void brick_geometry(int gw, int gh, int gd, int py, int px, int pz, int overlap, int rank, HostBrick &b);

// The per-frame set-up of one STATE: viewport, ray frame, per-brick clip
// planes, projected rectangles, first rays and composite order.  Fills
// everything in f except the LUT, the empty-cell flags, the output window
// and the counters.
int build_frame(int gw, int gh, int gd, int dtype, const HostBrick *bricks, int nb, const ivr_state &st,
                const ivr_render_params &p, FrameDesc &f, ivr_frame_info &info);

// colormap.c builders into hsize RGBA rows.
void build_colormap(int type, float *rgba, int hsize, float histmin, float histmax);

}  // namespace ivr
