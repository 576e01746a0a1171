"""Regenerates the recorded-animation fixtures in anim/.

Each anim/<name>.rsa holds every frame of one of the reference's recorded
animations (tests/unit_tests/silvers/<name>.sriv: the Renderer calls its
SerializingFactory records while a .riv artboard animates), converted by
rive_runtime_gb300.sriv into rive_scene.h recordings and packed with
sriv.pack_frames. They are the real content of the recorded-animation serving
workload (bench.py) and its tests. Draws with feathered paints and image draws
are left out. Needs the reference sources, so it runs only where they exist:

    python tests/golden/make_animations.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from conftest import load_package  # noqa: E402

load_package()
from rive_runtime_gb300 import sriv  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle  # noqa: E402

# name -> frame stride (1 = every frame)
ANIMATIONS = {
    "echo_show_demo": 1,          # 1024x884, clips and gradients
    "juice": 1,                   # 1080x1080
    "follow_path_animate_shape": 1,
    "collapsing_elements": 1,     # 1500x1500, 250 frames
    "layout_scroll_visibility": 1,
    "component_list_child_origin": 1,
    "hunter_x_demo": 8,           # 3387x1905, 130 clip paths per frame
}


def main():
    silvers = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests", "silvers")
    os.makedirs(os.path.join(HERE, "anim"), exist_ok=True)
    for name, stride in ANIMATIONS.items():
        with open(os.path.join(silvers, name + ".sriv"), "rb") as f:
            st = sriv.read_sriv(f.read())
        frames = [st.frame_scene(k)[0].to_bytes() for k in range(0, len(st.frames), stride)]
        data = sriv.pack_frames(frames)
        with open(os.path.join(HERE, "anim", name + ".rsa"), "wb") as f:
            f.write(data)
        print(f"{name}: {len(frames)} frames {st.width}x{st.height}, {len(data)} B")


if __name__ == "__main__":
    main()
