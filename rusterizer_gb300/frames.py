"""Render a benchmark workload a given number of times, synchronously (for profilers and quick
checks): one frame of configuration 0, 1 or 2 per repetition through the Renderer API, or a
batch of scenes of the scene mix through rast_render_batch.

  python -m rusterizer_gb300.frames --config 2 --frames 4
  python -m rusterizer_gb300.frames --mix 24 --tile 32 --heavy-entries 512 --frames 2

Prints the number of pipeline kernels the library launched (rast_kernel_launches), so that a
profiler's launch-skip count can be chosen.
"""
import argparse
import sys

import numpy as np

from . import _lib, renderer, scenes


def frames(config, n, tile=0, heavy_entries=0):
    sc = {0: scenes.config0, 1: scenes.config1, 2: scenes.config2}[config]()
    r = renderer.Renderer(sc["width"], sc["height"], sc.get("msaa", 4), tile=tile)
    _lib.check(_lib.load().rast_set_heavy_tile_entries(r._ctx, heavy_entries), "heavy tile entries")
    r.set_clear_depth(sc.get("clear_depth", np.finfo(np.float32).max))
    for i, t in enumerate(sc["textures"]):
        r.uniforms().bind_texture(i, renderer.Texture(t))
    blk = r.uniforms().write_block()
    blk.view, blk.projection = sc["view"], sc["proj"]
    for _ in range(n):
        for d in sc["draws"]:
            blk.world = d["world"]
            r.render(d, renderer.VS_MVP, d.get("fs", 0))
        r.framebuffer()
        if r.last_status not in (_lib.OK, _lib.TEXTURE_OOB):
            raise _lib.RastError(r.last_status, "framebuffer")
    r.close()


def mix(nscenes, n, tile=0, heavy_entries=0):
    from .batch import BatchRenderer
    sc = [scenes.batch_scene(s) for s in scenes.batch_scene_specs(nscenes, 3)]
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s, tile=tile)
    _lib.check(_lib.load().rast_set_heavy_tile_entries(br._ctx, heavy_entries), "heavy tile entries")
    outs = [np.zeros((s["height"], s["width"]), np.uint32) for s in sc]
    for _ in range(n):
        br.render(outs)
    br.close()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=2, choices=[0, 1, 2])
    ap.add_argument("--mix", type=int, default=0, help="render this many scenes of the batch mix instead")
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--heavy-entries", type=int, default=0)
    a = ap.parse_args(argv)
    if a.mix:
        mix(a.mix, a.frames, a.tile, a.heavy_entries)
    else:
        frames(a.config, a.frames, a.tile, a.heavy_entries)
    print("kernel launches:", _lib.load().rast_kernel_launches())
    return 0


if __name__ == "__main__":
    sys.exit(main())
