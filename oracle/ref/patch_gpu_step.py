"""Write the reference's EULERIAN_FLUID_SOLVER_2D.h with the GPU step members hooked in.

    python oracle/ref/patch_gpu_step.py REFERENCE_HEADER OUT_HEADER

This is the change INTEGRATION.md describes for a maintainer of the reference, applied
mechanically to a copy in the build directory (the reference's sources are read, never
edited): the solver gains a `GB2D_FLUID_STEP* gpu_step` member, and when it is set

  * AdvanceOneTimeStepThread(dt, tid)      EULERIAN_FLUID_SOLVER_2D.h:1140
  * CFLOneTimeStep()                       :3517
  * Levelset_Advection(dt, tid)            :1898
  * Reinitialization(dt, tid)              :2402
  * Velocity_Advection(dt, tid)            :1886
  * Projection(dt, tid)                    :2359

forward to the adapter (include/gb2d_adapter.hpp) and return; otherwise the reference's
own bodies run unchanged.  The headless driver built with REF_GPU (oracle/ref/Makefile,
target `gpu`) links the result against libgb2d.so.  Test infrastructure only.
"""
import sys

HOOKS = [
    ("\tvoid AdvanceOneTimeStepThread(const T& dt, const int& thread_id = 0)\n\t{\n",
     "\t\tif (gpu_step) { gpu_step->AdvanceOneTimeStepThread(dt, thread_id); return; }\n"),
    ("\tT CFLOneTimeStep(void)\n\t{\n",
     "\t\tif (gpu_step) { T d = gpu_step->CFLOneTimeStep(); c_f = gpu_step->c_f; g_f = gpu_step->g_f;\n"
     "\t\t                v_f = gpu_step->v_f; s_f = gpu_step->s_f; return d; }\n"),
    ("\tvoid Levelset_Advection(const T& dt, const int& thread_id)\n\t{\n",
     "\t\tif (gpu_step) { gpu_step->Levelset_Advection(dt, thread_id); return; }\n"),
    ("\tvoid Reinitialization(const T& dt, const int& thread_id)\n\t{\n",
     "\t\tif (gpu_step) { gpu_step->Reinitialization(dt, thread_id); return; }\n"),
    ("\tvoid Velocity_Advection(const T& dt, const int& thread_id)\n\t{\n",
     "\t\tif (gpu_step) { gpu_step->Velocity_Advection(dt, thread_id); return; }\n"),
    ("\tvoid Projection(const T& dt, const int& thread_id)\n\t{\n",
     "\t\tif (gpu_step) { gpu_step->Projection(dt, thread_id);\n"
     "\t\t                water_projection->max_velocity_x = gpu_step->max_velocity_x;\n"
     "\t\t                water_projection->max_velocity_y = gpu_step->max_velocity_y; return; }\n"),
]
MEMBER_AFTER = "\tADVECTION_2D*\t\t\t\t\tadvecting_field_variables;\n"
MEMBER = "\tGB2D_FLUID_STEP*\t\t\t\tgpu_step = 0;\t// the GPU path (gb2d); null: the reference's own code\n"
INCLUDE_AFTER = '#include "VISCOSITY_2D.h"\n'


def patch(text):
    def once(s, old, new):
        n = s.count(old)
        if n != 1:
            raise SystemExit(f"expected one occurrence of {old!r}, found {n}")
        return s.replace(old, new)
    text = text.replace("\r\n", "\n")
    text = once(text, INCLUDE_AFTER, INCLUDE_AFTER + '#include "gb2d_adapter.hpp"\n')
    text = once(text, MEMBER_AFTER, MEMBER_AFTER + MEMBER)
    for head, body in HOOKS:
        text = once(text, head, head + body)
    return text


if __name__ == "__main__":
    src, dst = sys.argv[1], sys.argv[2]
    with open(src, newline="") as f:
        out = patch(f.read())
    with open(dst, "w") as f:
        f.write(out)
