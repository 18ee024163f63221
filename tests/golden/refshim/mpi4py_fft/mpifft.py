"""Serial Transform chain and PFFT base class (single rank)."""
import numpy as np


class Transform:
    def __init__(self, xfftn, transfer, pencil):
        assert len(xfftn) == len(transfer) + 1 and len(pencil) == 2
        self._xfftn = tuple(xfftn)
        self._transfer = tuple(transfer)
        self._pencil = tuple(pencil)

    @property
    def input_array(self):
        return self._xfftn[0].input_array

    @property
    def output_array(self):
        return self._xfftn[-1].output_array

    @property
    def input_pencil(self):
        return self._pencil[0]

    @property
    def output_pencil(self):
        return self._pencil[1]

    def __call__(self, input_array=None, output_array=None, **kw):
        if input_array is not None:
            self.input_array[...] = input_array
        for i in range(len(self._transfer)):
            self._xfftn[i](**kw)
            arrayA = self._xfftn[i].output_array
            arrayB = self._xfftn[i + 1].input_array
            self._transfer[i](arrayA, arrayB)
        self._xfftn[-1](**kw)
        if output_array is not None:
            output_array[...] = self.output_array
            return output_array
        return self.output_array


class PFFT:
    def shape(self, forward_output=False):
        if forward_output:
            return self.forward.output_array.shape
        return self.forward.input_array.shape

    def local_slice(self, forward_output=True):
        shp = self.shape(forward_output)
        return tuple(slice(0, n) for n in shp)

    def dtype(self, forward_output=False):
        if forward_output:
            return self.forward.output_array.dtype
        return self.forward.input_array.dtype

    @property
    def dimensions(self):
        return len(self.forward.input_array.shape)

    def destroy(self):
        pass
