// thrust/async was removed in CCCL 3; the reference includes it but uses nothing from it.
#pragma once
